/*
 * engine.cu -- the GPU engine behind pcagb_solve, pcagb_solve_batch,
 * pcagb_complete and the GPU-backed search_exhaustive_complete of the libpca
 * ABI.
 *
 * Iterative deepening over the kernel length K, as in the reference's
 * tools/enumerate.c:624-662 and gpu/hybrid.cu:699-824, restructured for one
 * GB300 and for many tasks at once:
 *   - a batch of tasks shares every launch: level d holds the distinct
 *     states of all tasks still searched, each state tagged with its task;
 *   - levels 1..S are built breadth-first on the device, each deduplicated
 *     by the exact OEP table and kept in HBM in DFS order (levels do not
 *     depend on K, so each is built once per batch, not once per K);
 *   - the remaining K-S <= 3 instructions are enumerated by the suffix
 *     kernel, which takes the role of gpu/hybrid.cu:163-275;
 *   - a task leaves the search (its states are skipped) once its optimal
 *     depth is proven or its depth limit is reached;
 *   - the host only reads back sizes, per-task histograms, counters and the
 *     solving records.
 * Device memory comes from one arena allocated at engine creation: levels
 * grow from the bottom, per-expansion scratch (hash table, bitmap, scan
 * buffers) from the top, so a solve performs no cudaMalloc.
 */
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <functional>
#include <mutex>
#include <string>
#include <unordered_set>
#include <vector>

#include "../../include/pca_gb300.h"
#include "engine_kernels.cuh"
#include "gen_tables.h"

namespace pcagb {

static thread_local std::string g_err;

static void set_err(const char *fmt, ...)
{
    char b[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(b, sizeof b, fmt, ap);
    va_end(ap);
    g_err = b;
}

#define CK(call)                                                                       \
    do {                                                                               \
        cudaError_t e_ = (call);                                                       \
        if (e_ != cudaSuccess) {                                                       \
            set_err("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                    __LINE__);                                                         \
            return PCAGB_ECUDA;                                                        \
        }                                                                              \
    } while (0)

constexpr int kMaxBatch = 8192;
/* engine_init's budget for an engine whose arena each solve supplies */
constexpr size_t kArenaExternal = ~size_t(0);
/* slots of the pinned host buffer */
constexpr int kPinStatus = 0, kPinSurvivors = 1, kPinTotal = 2, kPinCount = 3, kPinFirst = 4,
              kPinHist = 64;
/* A level whose children's states fit in this many bytes, or in an eighth
   of the arena's free space, is written into space for all of them, so its
   build needs one host round trip instead of three. */
constexpr uint64_t kOneSyncBytes = 64ull << 20;
/* ordered solves with an automatic split (see run_batch) */
constexpr double kOrderMinStageMs = 2.0;
constexpr double kOrderStageShare = 0.1;
constexpr double kOrderMaxOverhead = 1.02;

struct Level {
    uint64_t n = 0;
    uint16_t *regs = nullptr;
    uint8_t *flags = nullptr;
    uint8_t *live = nullptr;
    uint16_t *task = nullptr;
    uint32_t *parent = nullptr;
    uint16_t *cidx = nullptr;
    uint8_t *rdl = nullptr;         /* register each state's last instruction wrote */
    uint8_t *own = nullptr;         /* dead-able older writes (engine_kernels.cuh) */
    uint8_t *twin = nullptr;        /* later member of a flag-twin class (k_twins) */
    uint16_t *probe = nullptr;      /* [n][8][4] r0..r7 on the first four tests (64 bytes:
                                       what a lane-per-prefix scan reads) */
    uint32_t *fcr = nullptr;        /* [n][8] rank of the first kept child writing r (set
                                       when the level below is materialised) */
    uint64_t *child_off = nullptr;  /* set when this level is expanded */
    uint64_t children = 0;
    std::vector<uint64_t> hist;     /* [task][128] states per liveness mask */
    bool lean = false;              /* k_materialize_probe wrote it: links and probes
                                       only (regs and flags unwritten) */
};

struct PathGather {
    const uint32_t *parent[SEARCH_MAX_DEPTH + 1];
    const uint16_t *cidx[SEARCH_MAX_DEPTH + 1];
    const uint16_t *task;           /* task of the level-S states */
};

/* For each record, the candidate indices of its prefix path and its task. */
__global__ void k_gather_paths(PathGather G, int S, const ulonglong2 *rec, uint64_t n,
                               uint16_t *out, uint16_t *task_out)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t q = rec[i].x;
        task_out[i] = G.task[q];
        for (int d = S; d >= 1; d--) {
            out[i * SEARCH_MAX_DEPTH + d - 1] = G.cidx[d][q];
            q = G.parent[d][q];
        }
    }
}

}  // namespace pcagb

using namespace pcagb;

struct pcagb_engine {
    int device = 0;
    int sms = 0;
    cudaStream_t stream = nullptr;
    char *arena = nullptr;
    size_t cap = 0, bottom = 0, top = 0;
    unsigned long long *d_small = nullptr;   /* [0] sol count [1] first [2] count
                                                [3] value-class evaluations run
                                                [4] the work counter of the insert and
                                                lean materialise kernels */
    uint32_t *d_status = nullptr;
    ulonglong2 *d_sol = nullptr;
    uint64_t sol_cap = 1u << 20;
    /* batch task table */
    int32_t *d_task_T = nullptr;
    uint32_t *d_task_target = nullptr;
    uint8_t *d_task_active = nullptr;
    uint16_t *d_task_io = nullptr;           /* [kMaxBatch][3][32] in0, in1, target */
    unsigned long long *d_hist = nullptr;    /* [kMaxBatch][128] */
    /* pinned host mirror of the small results (kPin* slots) and of d_hist:
       device-to-host reads of these never wait on their own */
    unsigned long long *h_pin = nullptr;
    std::vector<uint8_t> h_active;           /* host copy of d_task_active */
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr, ev3 = nullptr;
    cudaEvent_t evk0 = nullptr, evk1 = nullptr;   /* around a lane-per-prefix launch */
    int occ_insert = 4, occ_suffix = 8, occ_mat = 4, occ_lanes = 4,
        occ_mid_lanes = 4;   /* resident blocks per SM */
    uint64_t launches = 0;
    uint64_t h2d = 0, d2h = 0;
    uint64_t insert_launches = 0, suffix_launches = 0, insert_children = 0;
    uint64_t evals_run = 0;                  /* value-class evaluations the suffix kernels ran */
    float ms_insert = 0;
    double ms_lanes[PCAGB_MAXD] = {};        /* lane-per-prefix kernel device time per depth */
    /* autotuner: unit costs measured on this engine (running averages) */
    /* starting values: this engine's costs measured on a GB300 (one- and
       two-input depth-4 searches); every solve refines them */
    double t_child_ms = 1.8e-7;     /* device ms per child of a level build */
    double t_child_lean_ms = 1.2e-7; /* the same for a lean level (k_materialize_probe) */
    double t_build_fixed_ms = 0.08; /* device ms of a level build's fixed part */
    double t_eval_ms[4] = {0, 1.8e-9, 1.4e-9, 1.3e-9};  /* device ms per value-class
                                                           evaluation, per suffix depth */
    double dedup_ratio = 0.35;      /* survivors / children of the last build */
    /* launch choices of the suffix stages, with their measured costs (ms
       per value-class evaluation, running averages; n = stages measured) */
    double ft_ms[4][4] = {};        /* [suffix depth][tests checked per lane] */
    int ft_n[4][4] = {};
    double ck_ms[4][4] = {};        /* [suffix depth][index into kChunkChoices] */
    int ck_n[4][4] = {};
    double launch_rt_ms = 0.03;     /* host round trip of one launch of a chunked stage */
    int force_ft = 0, force_chunk = 0;   /* per solve: pcagb_opts_t overrides */
    bool measure = true;                 /* per solve: the GPU is its own (not
                                            shared_gpu), so its times are costs */
    int lean_K = -1;                     /* per solve: the last depth, whose stage
                                            reads its split level lean (-1: none) */

    /* per batch */
    std::vector<Level> levels;
    int ntasks = 0;
    int TPC = 32;
    bool no_oep = false;
    int max_feasible = SEARCH_MAX_DEPTH;
    TaskDev td{};
    float ms_expand = 0, ms_suffix = 0;

    void *alloc_bottom(size_t bytes)
    {
        bytes = (bytes + 255) & ~size_t(255);
        if (bottom + bytes > top) return nullptr;
        void *p = arena + bottom;
        bottom += bytes;
        return p;
    }
    void *alloc_top(size_t bytes)
    {
        bytes = (bytes + 255) & ~size_t(255);
        if (top < bottom + bytes) return nullptr;
        top -= bytes;
        return arena + top;
    }
    int grid(int per_sm = 4) const { return sms * per_sm; }
};

namespace {

/* Unit costs the engines of one device have measured (the autotuner's
   model), shared so that a new engine, e.g. a server's slot, starts from
   what earlier engines measured on the same GPU instead of the defaults. */
struct CostModel {
    bool set = false;
    double t_child_ms = 0, t_child_lean_ms = 0, t_build_fixed_ms = 0, t_eval_ms[4] = {0, 0, 0, 0},
           dedup_ratio = 0;
    double ft_ms[4][4] = {}, ck_ms[4][4] = {}, launch_rt_ms = 0.03;
    int ft_n[4][4] = {}, ck_n[4][4] = {};
};
std::mutex g_cost_mu;
CostModel g_cost[64];

void load_costs(pcagb_engine *e)
{
    std::lock_guard<std::mutex> lk(g_cost_mu);
    if (e->device < 0 || e->device >= 64 || !g_cost[e->device].set) return;
    const CostModel &c = g_cost[e->device];
    e->t_child_ms = c.t_child_ms;
    e->t_child_lean_ms = c.t_child_lean_ms;
    e->t_build_fixed_ms = c.t_build_fixed_ms;
    for (int i = 0; i < 4; i++) e->t_eval_ms[i] = c.t_eval_ms[i];
    e->dedup_ratio = c.dedup_ratio;
    memcpy(e->ft_ms, c.ft_ms, sizeof c.ft_ms);
    memcpy(e->ft_n, c.ft_n, sizeof c.ft_n);
    memcpy(e->ck_ms, c.ck_ms, sizeof c.ck_ms);
    memcpy(e->ck_n, c.ck_n, sizeof c.ck_n);
    e->launch_rt_ms = c.launch_rt_ms;
}

void store_costs(const pcagb_engine *e)
{
    std::lock_guard<std::mutex> lk(g_cost_mu);
    if (e->device < 0 || e->device >= 64) return;
    CostModel &c = g_cost[e->device];
    c.t_child_ms = e->t_child_ms;
    c.t_child_lean_ms = e->t_child_lean_ms;
    c.t_build_fixed_ms = e->t_build_fixed_ms;
    for (int i = 0; i < 4; i++) c.t_eval_ms[i] = e->t_eval_ms[i];
    c.dedup_ratio = e->dedup_ratio;
    memcpy(c.ft_ms, e->ft_ms, sizeof c.ft_ms);
    memcpy(c.ft_n, e->ft_n, sizeof c.ft_n);
    memcpy(c.ck_ms, e->ck_ms, sizeof c.ck_ms);
    memcpy(c.ck_n, e->ck_n, sizeof c.ck_n);
    c.launch_rt_ms = e->launch_rt_ms;
    c.set = true;
}

/* every host<->device copy of a solve goes through here and is counted */
cudaError_t e_copy(pcagb_engine *e, void *dst, const void *src, size_t n, cudaMemcpyKind kind,
                   cudaStream_t st)
{
    if (kind == cudaMemcpyHostToDevice) e->h2d += n;
    if (kind == cudaMemcpyDeviceToHost) e->d2h += n;
    return cudaMemcpyAsync(dst, src, n, kind, st);
}

int check_launch(pcagb_engine *e)
{
    e->launches++;
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) {
        set_err("kernel launch failed: %s", cudaGetErrorString(err));
        return PCAGB_ECUDA;
    }
    return PCAGB_OK;
}

/* Exclusive scan of a[0..n) in place; returns the total in *total, or,
   with total null, only enqueues the scan (scanning n + 1 entries whose last
   is 0 leaves the total on the device, in a[n]). */
int exclusive_scan(pcagb_engine *e, uint64_t *a, uint64_t n, uint64_t *total)
{
    if (n == 0) {
        if (total) *total = 0;
        return PCAGB_OK;
    }
    uint64_t nb = (n + kScanBlock - 1) / kScanBlock;
    size_t saved = e->top;
    uint64_t *sums = (uint64_t *)e->alloc_top((nb + 1) * sizeof(uint64_t));
    if (!sums) { set_err("arena exhausted in scan"); return PCAGB_ENOMEM; }
    k_scan_local<<<(unsigned)nb, 256, 0, e->stream>>>(a, n, sums);
    int rc = check_launch(e);
    if (rc) return rc;
    if (nb == 1) {
        if (total) {
            CK(e_copy(e, &e->h_pin[kPinTotal], sums, sizeof(uint64_t), cudaMemcpyDeviceToHost,
                      e->stream));
            CK(cudaStreamSynchronize(e->stream));
            *total = e->h_pin[kPinTotal];
        }
    } else {
        rc = exclusive_scan(e, sums, nb, total);
        if (rc) return rc;
        k_scan_add<<<(unsigned)nb, 256, 0, e->stream>>>(a, n, sums);
        rc = check_launch(e);
        if (rc) return rc;
    }
    e->top = saved;
    return PCAGB_OK;
}

LevelDev view(const Level &L)
{
    return LevelDev{L.regs, L.flags, L.live, L.task, L.child_off, L.n, L.rdl, L.parent, L.own,
                    L.twin, L.probe};
}

int alloc_level(pcagb_engine *e, Level &L, uint64_t n)
{
    L.n = n;
    L.regs = (uint16_t *)e->alloc_bottom(n * 8 * e->TPC * 2);
    L.flags = (uint8_t *)e->alloc_bottom(n * e->TPC);
    L.live = (uint8_t *)e->alloc_bottom(n);
    L.task = (uint16_t *)e->alloc_bottom(n * 2);
    L.parent = (uint32_t *)e->alloc_bottom(n * 4);
    L.cidx = (uint16_t *)e->alloc_bottom(n * 2);
    L.rdl = (uint8_t *)e->alloc_bottom(n);
    L.own = (uint8_t *)e->alloc_bottom(n);
    L.twin = (uint8_t *)e->alloc_bottom(n);
    L.probe = (uint16_t *)e->alloc_bottom(n * 64);
    if (!L.regs || !L.flags || !L.live || !L.task || !L.parent || !L.cidx || !L.rdl || !L.own ||
        !L.twin || !L.probe)
        return PCAGB_ENOMEM;
    return PCAGB_OK;
}

/* Enqueue the level's (task, mask) histogram and its copy into the pinned
   buffer; take_hist reads it after the stream has been synchronised. With
   n_dev set, L.n is an upper bound and the device holds the count. */
int enqueue_hist(pcagb_engine *e, const Level &L, const unsigned long long *n_dev)
{
    const size_t nh = (size_t)e->ntasks * 128;
    CK(cudaMemsetAsync(e->d_hist, 0, nh * sizeof(unsigned long long), e->stream));
    if (nh <= 4096)
        k_task_hist_smem<<<e->grid(2), 256, nh * sizeof(uint32_t), e->stream>>>(
            L.live, L.task, L.n, n_dev, (uint32_t)nh, e->d_hist);
    else
        k_task_hist<<<e->grid(2), 256, 0, e->stream>>>(L.live, L.task, L.n, n_dev, e->d_hist);
    int rc = check_launch(e);
    if (rc) return rc;
    CK(e_copy(e, e->h_pin + kPinHist, e->d_hist, nh * sizeof(uint64_t), cudaMemcpyDeviceToHost,
              e->stream));
    return PCAGB_OK;
}

void take_hist(pcagb_engine *e, Level &L)
{
    const size_t nh = (size_t)e->ntasks * 128;
    L.hist.assign(e->h_pin + kPinHist, e->h_pin + kPinHist + nh);
}

/* log2 of the slices each parent's candidates are cut into, so that a
   level of few parents still gives every resident warp work (up to 32
   slices; 1 slice once the parents alone fill the grid) */
uint32_t split_log2(uint64_t parents, int grid)
{
    const uint64_t warps = (uint64_t)grid * kWarpsPerBlock;
    uint32_t l = 0;
    while (l < 5 && (parents << (l + 1)) <= warps) l++;
    return l;
}

template <int TPC>
int launch_expand(pcagb_engine *e, const Level &P, const uint32_t *fcr_up,
                  unsigned long long *table, uint64_t tmask)
{
    const int g = e->grid(e->occ_insert);
    /* the work-item counter the kernel's warps draw from */
    uint32_t *next = reinterpret_cast<uint32_t *>(e->d_small + 4);
    CK(cudaMemsetAsync(next, 0, 4, e->stream));
    k_expand_insert<TPC><<<g, kThreads, 0, e->stream>>>(view(P), e->td, table, tmask,
                                                        e->d_status, split_log2(P.n, g), fcr_up,
                                                        next);
    return check_launch(e);
}

template <int TPC>
int launch_materialize(pcagb_engine *e, const Level &P, const uint32_t *fcr_up,
                       const uint32_t *bitmap, const uint64_t *word_off, Level &C)
{
    LevelOut out{C.regs, C.flags, C.live, C.task, C.parent, C.cidx, C.rdl, C.own, C.probe};
    const int g = e->grid(e->occ_mat);
    if (C.lean) {
        uint32_t *next = reinterpret_cast<uint32_t *>(e->d_small + 4);
        CK(cudaMemsetAsync(next, 0, 4, e->stream));
        k_materialize_probe<TPC><<<g, kThreads, 0, e->stream>>>(view(P), e->td, bitmap, word_off,
                                                                out, split_log2(P.n, g), fcr_up,
                                                                next);
    } else
        k_materialize<TPC><<<g, kThreads, 0, e->stream>>>(view(P), e->td, bitmap, word_off, out,
                                                          split_log2(P.n, g), P.fcr, fcr_up);
    return check_launch(e);
}

/* Build level d+1 from level d for the active tasks. Returns PCAGB_ENOMEM
 * (and leaves the arena as it was) when the level does not fit.
 *
 * The child count comes from the parent level's histogram on the host (the
 * same sum the device scan forms), so nothing waits before the insert. A
 * level whose children's states fit in kOneSyncBytes or an eighth of the
 * free arena is materialised into space for every child and its survivor
 * count, status, scan total and histogram come back in one round trip; a
 * larger level reads the survivor count first and allocates exactly. */
int build_level(pcagb_engine *e, int d, bool lean = false)
{
    const GenTables &gt = gen_tables();
    Level &P = e->levels[d];
    const size_t bottom0 = e->bottom, top0 = e->top;
    auto fail = [&](int rc) {
        e->bottom = bottom0;
        e->top = top0;
        if (rc == PCAGB_ENOMEM) {
            P.child_off = nullptr;
            P.fcr = nullptr;
        }
        return rc;
    };
    if (!P.child_off) {
        P.child_off = (uint64_t *)e->alloc_bottom((P.n + 1) * sizeof(uint64_t));
        if (!P.child_off) return fail(PCAGB_ENOMEM);
        CK(cudaMemsetAsync(P.child_off + P.n, 0, sizeof(uint64_t), e->stream));
        k_child_counts<<<e->grid(2), 256, 0, e->stream>>>(P.live, P.task, e->td.active, P.n,
                                                          P.child_off);
        int rc = check_launch(e);
        if (rc) return rc;
        rc = exclusive_scan(e, P.child_off, P.n + 1, nullptr);
        if (rc) return fail(rc);
        uint64_t c = 0;
        for (size_t i = 0; i < P.hist.size(); i++)
            if (e->h_active[i >> 7]) c += P.hist[i] * (uint64_t)gt.nc((int)(i & 127));
        P.children = c;
    }
    if (!P.fcr && !e->no_oep) {
        P.fcr = (uint32_t *)e->alloc_bottom(P.n * 8 * sizeof(uint32_t));
        if (!P.fcr) return fail(PCAGB_ENOMEM);
        CK(cudaMemsetAsync(P.fcr, 0xFF, P.n * 8 * sizeof(uint32_t), e->stream));
    }
    /* the dead-write rule of the insert kernel needs the first-child ranks
       of the level above (unset at the root) */
    const uint32_t *fcr_up = d >= 1 ? e->levels[d - 1].fcr : nullptr;
    const uint64_t children = P.children;
    if (children >= (1ull << 38)) return fail(PCAGB_ENOMEM);
    const uint64_t words = (children + 31) / 32;
    const uint64_t state_bytes = 8ull * 2 * e->TPC + e->TPC + 1 + 2 + 4 + 2 + 1 + 1 + 1 + 64;
    const bool one_sync =
        children * state_bytes <= std::max<uint64_t>(kOneSyncBytes, (e->top - e->bottom) / 8);

    cudaEventRecord(e->ev0, e->stream);
    uint32_t *bitmap = (uint32_t *)e->alloc_top(words * 4 + 4);
    if (!bitmap) return fail(PCAGB_ENOMEM);
    uint64_t survivors = children;
    if (e->no_oep) {
        k_mark_all<<<e->grid(2), 256, 0, e->stream>>>(bitmap, words, children);
        int rc = check_launch(e);
        if (rc) return rc;
    } else {
        if (P.n >= (1ull << 28)) return fail(PCAGB_ENOMEM);
        /* mark the later flag twins of the parent level (k_twins); their
           table lives on the scratch side only while the pass runs (stream
           order keeps the space from being reused before it ends) */
        CK(cudaMemsetAsync(P.twin, 0, P.n, e->stream));
        if (P.n >= 2) {
            const size_t top_tw = e->top;
            uint64_t tslots = 1024;
            while (tslots < 2 * P.n) tslots <<= 1;
            unsigned long long *tt = (unsigned long long *)e->alloc_top(tslots * 8);
            if (!tt) return fail(PCAGB_ENOMEM);
            CK(cudaMemsetAsync(tt, 0, tslots * 8, e->stream));
            if (e->TPC == 16)
                k_twins<16><<<e->grid(4), 256, 0, e->stream>>>(view(P), e->td, tt, tslots - 1,
                                                              P.twin, e->d_status);
            else
                k_twins<32><<<e->grid(4), 256, 0, e->stream>>>(view(P), e->td, tt, tslots - 1,
                                                              P.twin, e->d_status);
            const int rct = check_launch(e);
            if (rct) return rct;
            e->top = top_tw;
        }
        uint64_t slots = 1024;
        while (slots < 2 * children) slots <<= 1;
        unsigned long long *table = (unsigned long long *)e->alloc_top(slots * 8);
        if (!table) return fail(PCAGB_ENOMEM);
        CK(cudaMemsetAsync(table, 0, slots * 8, e->stream));
        CK(cudaMemsetAsync(bitmap, 0, words * 4 + 4, e->stream));
        CK(cudaMemsetAsync(e->d_small + 2, 0, 8, e->stream));
        cudaEventRecord(e->ev2, e->stream);
        int rc = e->TPC == 16 ? launch_expand<16>(e, P, fcr_up, table, slots - 1)
                              : launch_expand<32>(e, P, fcr_up, table, slots - 1);
        if (rc) return rc;
        cudaEventRecord(e->ev3, e->stream);
        k_mark<<<e->grid(4), 256, 0, e->stream>>>(table, slots, P.child_off, bitmap,
                                                  e->d_small + 2);
        rc = check_launch(e);
        if (rc) return rc;
        CK(e_copy(e, &e->h_pin[kPinStatus], e->d_status, 4, cudaMemcpyDeviceToHost, e->stream));
        CK(e_copy(e, &e->h_pin[kPinSurvivors], e->d_small + 2, 8, cudaMemcpyDeviceToHost,
                  e->stream));
        if (!one_sync) {
            CK(cudaStreamSynchronize(e->stream));
            if ((uint32_t)e->h_pin[kPinStatus]) {
                set_err("expansion of level %d hit a device limit (status %u)", d + 1,
                        (uint32_t)e->h_pin[kPinStatus]);
                return PCAGB_ELIMIT;
            }
            survivors = e->h_pin[kPinSurvivors];
        }
        e->insert_launches++;
        e->insert_children += children;
    }
    uint64_t *word_off = (uint64_t *)e->alloc_top((words + 1) * sizeof(uint64_t));
    if (!word_off) return fail(PCAGB_ENOMEM);
    CK(cudaMemsetAsync(word_off + words, 0, sizeof(uint64_t), e->stream));
    k_popc<<<e->grid(2), 256, 0, e->stream>>>(bitmap, words, word_off);
    int rc = check_launch(e);
    if (rc) return rc;
    rc = exclusive_scan(e, word_off, words + 1, nullptr);
    if (rc) return fail(rc);
    CK(e_copy(e, &e->h_pin[kPinTotal], word_off + words, 8, cudaMemcpyDeviceToHost, e->stream));
    if (!one_sync) {
        /* the winners' ranks must stay inside the level about to be sized */
        CK(cudaStreamSynchronize(e->stream));
        if (e->h_pin[kPinTotal] != survivors) {
            set_err("internal: bitmap holds %llu winners, table %llu",
                    (unsigned long long)e->h_pin[kPinTotal], (unsigned long long)survivors);
            return PCAGB_ELIMIT;
        }
    }
    Level C;
    C.lean = lean;
    /* one round trip: space for every child (the ranks of the marked
       children are below their count, whatever the table did) */
    const uint64_t space = one_sync ? children : survivors;
    if (space >= (1ull << 28)) return fail(PCAGB_ENOMEM);
    if (alloc_level(e, C, space) != PCAGB_OK) return fail(PCAGB_ENOMEM);
    rc = e->TPC == 16 ? launch_materialize<16>(e, P, fcr_up, bitmap, word_off, C)
                      : launch_materialize<32>(e, P, fcr_up, bitmap, word_off, C);
    if (rc) return rc;
    cudaEventRecord(e->ev1, e->stream);
    rc = enqueue_hist(e, C, one_sync && !e->no_oep ? e->d_small + 2 : nullptr);
    if (rc) return rc;
    CK(cudaStreamSynchronize(e->stream));
    if (one_sync && !e->no_oep) {
        if ((uint32_t)e->h_pin[kPinStatus]) {
            set_err("expansion of level %d hit a device limit (status %u)", d + 1,
                    (uint32_t)e->h_pin[kPinStatus]);
            return fail(PCAGB_ELIMIT);
        }
        survivors = e->h_pin[kPinSurvivors];
        if (e->h_pin[kPinTotal] != survivors) {
            set_err("internal: bitmap holds %llu winners, table %llu",
                    (unsigned long long)e->h_pin[kPinTotal], (unsigned long long)survivors);
            return fail(PCAGB_ELIMIT);
        }
        C.n = survivors;
    }
    take_hist(e, C);
    if (!e->no_oep) {
        float ims = 0;
        cudaEventElapsedTime(&ims, e->ev2, e->ev3);
        e->ms_insert += ims;
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, e->ev0, e->ev1);
    e->ms_expand += ms;
    e->top = top0;
    if (!e->measure) {
        /* a shared GPU: the build's time is the mix's, not a cost */
    } else if (children > 100000) {
        const double per = std::max(0.0, (ms - e->t_build_fixed_ms) / (double)children);
        double &t = lean ? e->t_child_lean_ms : e->t_child_ms;
        t = 0.7 * t + 0.3 * per;
        if (!e->no_oep) e->dedup_ratio = 0.7 * e->dedup_ratio + 0.3 * ((double)survivors / children);
    } else if (children > 0) {
        e->t_build_fixed_ms = 0.7 * e->t_build_fixed_ms + 0.3 * ms;
    }
    e->levels.push_back(std::move(C));
    return PCAGB_OK;
}

struct RawSol {
    std::vector<uint16_t> kernel;  /* kernel instructions */
    uint32_t out_reg = 0;
    std::vector<uint32_t> key;     /* DFS-order key: candidate indices */
};

/* One task of a batch, host side. */
struct TaskRun {
    search_state_t root;           /* level-0 state */
    int T = 0;
    uint16_t target[MAX_TESTS] = {};
    std::vector<int> order;        /* device test order */
    int max_depth = 0, min_depth = 0;
    bool done = false;
    int optimal_depth = -1;
    uint64_t nrec = 0;
    std::vector<RawSol> sols;
    double t_done = 0;
    pcagb_result_t res{};
};

/* Visiting order of a suffix stage: a permutation of the level's prefixes
 * (null = DFS order), processed `chunk` prefixes in the first launch and
 * twice as many in each next one; with stop_at_first the stage ends after
 * the first launch that found a solution. Reports how far it got. */
struct StageOrder {
    const uint32_t *order = nullptr;
    uint64_t chunk = 0;
    bool stop_at_first = false;
    uint64_t prefixes_to_first = 0;
    float ms_to_first = 0;
};

/* Turn solving records r0..r1 of the stage at depth K from level S into
 * the tasks' raw solutions (kept sorted in DFS order). `first` is the
 * packed DFS-first key, used instead of the records for one task in
 * first-only mode. */
int take_records(pcagb_engine *e, int S, int K, std::vector<TaskRun> &runs, bool first_only,
                 uint64_t r0, uint64_t r1, unsigned long long first)
{
    const GenTables &gt = gen_tables();
    const Level &L = e->levels[S];
    const int s = K - S;
    std::vector<ulonglong2> rec;
    if (first_only && e->ntasks == 1) {
        const uint64_t m1 = (first >> 24) & 4095, m2 = (first >> 12) & 4095, fc = first & 4095;
        /* low 16 bits with bit 15 set: a candidate index, not a class */
        rec.push_back(make_ulonglong2(first >> 36, (m1 << 32) | (m2 << 16) | (0x8000u | fc)));
    } else {
        if (r1 > e->sol_cap) {
            set_err("%llu solving records exceed the buffer of %llu", (unsigned long long)r1,
                    (unsigned long long)e->sol_cap);
            return PCAGB_ELIMIT;
        }
        rec.resize(r1 - r0);
        CK(e_copy(e, rec.data(), e->d_sol + r0, rec.size() * sizeof(ulonglong2),
                  cudaMemcpyDeviceToHost, e->stream));
        CK(cudaStreamSynchronize(e->stream));
    }
    std::vector<uint16_t> paths(rec.size() * SEARCH_MAX_DEPTH, 0);
    std::vector<uint16_t> rtask(rec.size(), 0);
    {
        const size_t top0 = e->top;
        ulonglong2 *d_rec = (ulonglong2 *)e->alloc_top(rec.size() * sizeof(ulonglong2));
        uint16_t *d_paths = (uint16_t *)e->alloc_top(paths.size() * 2);
        uint16_t *d_task = (uint16_t *)e->alloc_top(rtask.size() * 2);
        if (!d_rec || !d_paths || !d_task) {
            set_err("arena exhausted gathering paths");
            return PCAGB_ENOMEM;
        }
        CK(e_copy(e, d_rec, rec.data(), rec.size() * sizeof(ulonglong2), cudaMemcpyHostToDevice,
                  e->stream));
        PathGather G{};
        for (int d = 1; d <= S; d++) {
            G.parent[d] = e->levels[d].parent;
            G.cidx[d] = e->levels[d].cidx;
        }
        G.task = L.task;
        k_gather_paths<<<64, 256, 0, e->stream>>>(G, S, d_rec, rec.size(), d_paths, d_task);
        int rc = check_launch(e);
        if (rc) return rc;
        CK(e_copy(e, paths.data(), d_paths, paths.size() * 2, cudaMemcpyDeviceToHost, e->stream));
        CK(e_copy(e, rtask.data(), d_task, rtask.size() * 2, cudaMemcpyDeviceToHost, e->stream));
        CK(cudaStreamSynchronize(e->stream));
        e->top = top0;
    }
    std::vector<uint8_t> touched(runs.size(), 0);
    for (size_t i = 0; i < rec.size(); i++) {
        TaskRun &tr = runs[rtask[i]];
        touched[rtask[i]] = 1;
        tr.nrec++;
        RawSol base;
        uint32_t mask = (tr.root.live >> 1) & 127u;
        auto take = [&](uint32_t c) {
            const uint32_t idx = gt.cand_off[mask] + c;
            base.kernel.push_back(gt.cand[idx]);
            base.key.push_back(c);
            mask |= 1u << (UOP_RD(gt.cand_uop[idx]) - 1);
        };
        for (int d = 0; d < S; d++) take(paths[i * SEARCH_MAX_DEPTH + d]);
        const uint32_t m1 = (uint32_t)(rec[i].y >> 32), m2 = (uint32_t)((rec[i].y >> 16) & 0xFFFF);
        const uint32_t low = (uint32_t)(rec[i].y & 0xFFFF);
        if (s >= 2) take(m1);
        if (s >= 3) take(m2);
        if (s == 0) {
            base.out_reg = low;
            base.key.push_back(0);
            tr.sols.push_back(base);
            continue;
        }
        if (low & 0x8000u) {
            RawSol r = base;
            const uint32_t c = low & 0x7FFF;
            const uint32_t idx = gt.cand_off[mask] + c;
            r.kernel.push_back(gt.cand[idx]);
            r.key.push_back(c);
            r.out_reg = UOP_RD(gt.cand_uop[idx]);
            tr.sols.push_back(r);
            continue;
        }
        for (uint32_t c = 0; c < (uint32_t)gt.nc(mask); c++) {
            const uint32_t idx = gt.cand_off[mask] + c;
            if (gt.cand_vc[idx] != low) continue;
            RawSol r = base;
            r.kernel.push_back(gt.cand[idx]);
            r.key.push_back(c);
            r.out_reg = UOP_RD(gt.cand_uop[idx]);
            tr.sols.push_back(r);
        }
    }
    for (size_t t = 0; t < runs.size(); t++)
        if (touched[t])
            std::sort(runs[t].sols.begin(), runs[t].sols.end(),
                      [](const RawSol &a, const RawSol &b) { return a.key < b.key; });
    return PCAGB_OK;
}

/* Work-item shapes of the suffix kernels, by suffix depth (index 0 is
   unused): at depth 1 the prefixes a warp scans at once (1: a warp per
   prefix, k_suffix; 32: a lane per prefix, k_suffix_lanes); at depths 2
   and 3 the middle-instruction chunk a warp-per-item work item takes, or
   kLaneShape: a lane per innermost middle (k_suffix_mid_lanes). */
constexpr uint32_t kLaneShape = 1024;
constexpr uint32_t kChunkChoices[4][4] = {
    {1, 1, 1, 1}, {1, 32, 1, 32}, {8, 16, 32, kLaneShape}, {1, 2, 4, kLaneShape}};
constexpr int kChunkOptions[4] = {1, 2, 4, 4};
/* below this many prefixes a level gives a lane-per-prefix launch fewer
   warps than the SMs hold: the depth-1 default is then a warp per prefix */
constexpr uint64_t kLanesMinPrefixes = 32ull * 152 * 4;
/* A stage is large enough to measure a launch choice on; each choice is
   measured this many times before the cheapest is kept. */
constexpr uint64_t kTuneMinEvals = 20000000ull;
constexpr int kTuneSamples = 2;

/* The option to use among n with measured costs ms[i] (n_meas[i] stages):
   an unmeasured one first when exploring, else the cheapest measured; def
   when none is measured. */
int pick_option(const double *ms, const int *n_meas, int n, int def, bool explore)
{
    if (explore)
        for (int round = 1; round <= kTuneSamples; round++)
            for (int i = 0; i < n; i++)
                if (n_meas[i] < round) return i;
    int best = -1;
    for (int i = 0; i < n; i++)
        if (n_meas[i] > 0 && (best < 0 || ms[i] < ms[best])) best = i;
    return best < 0 ? def : best;
}

void record_cost(double &ms, int &n, double v)
{
    ms = n == 0 ? v : 0.7 * ms + 0.3 * v;
    n++;
}

template <int TPC>
void launch_suffix_lanes(int ft, int g, cudaStream_t st, const LevelDev &L, const TaskDev &td,
                         const SolBuf &sb, const PrefixRange &R, const LeanDev &lean)
{
    if (ft == 1) k_suffix_lanes<TPC, 1><<<g, kThreads, 0, st>>>(L, td, sb, R, lean);
    else if (ft == 3) k_suffix_lanes<TPC, 3><<<g, kThreads, 0, st>>>(L, td, sb, R, lean);
    else k_suffix_lanes<TPC, 2><<<g, kThreads, 0, st>>>(L, td, sb, R, lean);
}

template <int TPC, int SD>
void launch_mid_lanes(int ft, int g, cudaStream_t st, const LevelDev &L, const TaskDev &td,
                      const SolBuf &sb, uint32_t cpp, const PrefixRange &R)
{
    if (ft == 1) k_suffix_mid_lanes<TPC, SD, 1><<<g, kThreads, 0, st>>>(L, td, sb, cpp, R);
    else if (ft == 3) k_suffix_mid_lanes<TPC, SD, 3><<<g, kThreads, 0, st>>>(L, td, sb, cpp, R);
    else k_suffix_mid_lanes<TPC, SD, 2><<<g, kThreads, 0, st>>>(L, td, sb, cpp, R);
}

template <int TPC, int SD>
void launch_suffix(int ft, int g, cudaStream_t st, const LevelDev &L, const TaskDev &td,
                   const SolBuf &sb, uint32_t cpp, uint32_t chunk, const PrefixRange &R)
{
    if (ft == 1) k_suffix<TPC, SD, 1><<<g, kThreads, 0, st>>>(L, td, sb, cpp, chunk, R);
    else if (ft == 3) k_suffix<TPC, SD, 3><<<g, kThreads, 0, st>>>(L, td, sb, cpp, chunk, R);
    else k_suffix<TPC, SD, 2><<<g, kThreads, 0, st>>>(L, td, sb, cpp, chunk, R);
}

/* Run the last stage at depth K from level S (suffix depth K-S, or the leaf
 * check when K == S) for the active tasks; appends each task's raw
 * solutions in DFS order.
 *
 * With several active tasks and `on_tasks` given, the suffix stage runs as
 * consecutive launches over groups of whole tasks (a level holds its tasks'
 * states task after task), each group about 1.5 ms of work, and calls
 * on_tasks(lo, hi) once tasks lo..hi-1 are searched at this depth, their
 * solutions taken: a batch's tasks are decided one group after another
 * instead of all at the end of the stage. */
int run_stage(pcagb_engine *e, int S, int K, std::vector<TaskRun> &runs, bool first_only,
              StageOrder *so = nullptr,
              const std::function<void(int, int)> *on_tasks = nullptr)
{
    const GenTables &gt = gen_tables();
    Level &L = e->levels[S];
    const int s = K - S;
    CK(cudaMemsetAsync(e->d_small, 0, 8, e->stream));
    CK(cudaMemsetAsync(e->d_small + 1, 0xFF, 8, e->stream));
    SolBuf sb{e->d_small, e->d_sol, e->sol_cap, e->d_small + 1, e->d_small + 3};
    int tuned_ft = 0, tuned_ck = -1;   /* the launch choices this stage used */
    int lane_launches = 0;             /* lane-per-prefix launches of this stage */
    /* launch choices are explored and timed on single-task stages only: a
       batch's stage mixes tasks (and, in a server, shares the GPU with
       other solves), so its times would not compare choices */
    int nact_stage = 0;
    for (size_t i = 0; i < e->h_active.size(); i++) nact_stage += e->h_active[i] ? 1 : 0;
    bool stopped_early = false;
    cudaEventRecord(e->ev0, e->stream);
    const bool t16 = e->TPC == 16;
    const int g = e->grid(e->occ_suffix);
    int rc = PCAGB_OK;
    uint64_t taken = 0;  /* records already turned into solutions */
    if (s == 0) {
        if (t16) k_leaf<16><<<e->grid(4), 256, 0, e->stream>>>(view(L), e->td, sb);
        else k_leaf<32><<<e->grid(4), 256, 0, e->stream>>>(view(L), e->td, sb);
        rc = check_launch(e);
        if (rc) return rc;
    } else if (s <= 3) {
        int ncmax = 0;
        uint64_t evals_pred = 0;
        for (size_t i = 0; i < L.hist.size(); i++)
            if (L.hist[i]) {
                ncmax = std::max(ncmax, gt.nc((int)(i & 127)));
                if (e->h_active[i >> 7]) evals_pred += L.hist[i] * gt.ev[s][i & 127];
            }
        /* launch choices: forced by the caller, else the cheapest measured
           (an unmeasured one is tried first on a stage large enough) */
        const bool explore = evals_pred >= kTuneMinEvals && !so && nact_stage == 1 && e->measure;
        int ft = e->force_ft;
        if (ft < 1 || ft > 3) ft = 1 + pick_option(&e->ft_ms[s][1], &e->ft_n[s][1], 3, 1, explore);
        int ck = -1;
        uint32_t chunk = 1;
        /* a lane per prefix needs every prefix's last write: not at the root */
        const bool lanes_ok = s == 1 && S >= 1;
        if (L.lean) {
            /* a lean level holds no register block: a lane per prefix */
            ck = 1;
            chunk = 32;
        } else if (s >= 2 || lanes_ok) {
            if (e->force_chunk >= 1) {
                chunk = s == 1 ? (e->force_chunk >= 32 ? 32u : 1u)
                        : e->force_chunk == (int)kLaneShape ? kLaneShape
                                                             : (uint32_t)std::min(e->force_chunk, 64);
            } else {
                /* shapes are explored once the tests-per-lane choice is */
                const bool ft_done = e->ft_n[s][1] >= kTuneSamples &&
                                     e->ft_n[s][2] >= kTuneSamples && e->ft_n[s][3] >= kTuneSamples;
                /* unmeasured, the lane shapes: a stage that is not timed
                   (an ordered or chunked first-only stage, or one too small
                   to explore on) keeps its default, and the lanes measured
                   2.3-3x faster on every stage that was timed; at depth 1 a
                   level too small to fill the GPU with 32 prefixes a warp
                   stays a warp per prefix */
                const int def = s == 1 ? (L.n >= kLanesMinPrefixes ? 1 : 0) : 3;
                ck = pick_option(e->ck_ms[s], e->ck_n[s], kChunkOptions[s], def,
                                 explore && ft_done);
                chunk = kChunkChoices[s][ck];
            }
        }
        /* work items per prefix: one (depth 1); the middle chunks; with a
           lane per middle, 32 first middles (depth 2) or one (depth 3) */
        const uint32_t cpp =
            s == 1                ? 1u
            : chunk == kLaneShape ? std::max(1u, s == 2 ? (uint32_t)(ncmax + 31) / 32
                                                        : (uint32_t)ncmax)
                                  : std::max(1u, (uint32_t)((ncmax + chunk - 1) / chunk));
        auto launch = [&](const PrefixRange &R) {
            const LevelDev V = view(L);
            if (s == 1) {
                const bool lanes = chunk == 32;
                if (lanes) {
                    const int gl = e->grid(e->occ_lanes);
                    LeanDev lean{nullptr, nullptr, nullptr};
                    if (L.lean)
                        lean = LeanDev{e->levels[S - 1].regs, e->levels[S - 1].live, L.cidx};
                    /* the kernel's own device time (without the count pass) */
                    cudaEventRecord(e->evk0, e->stream);
                    if (t16) launch_suffix_lanes<16>(ft, gl, e->stream, V, e->td, sb, R, lean);
                    else launch_suffix_lanes<32>(ft, gl, e->stream, V, e->td, sb, R, lean);
                    cudaEventRecord(e->evk1, e->stream);
                    lane_launches++;
                } else {
                    if (t16) launch_suffix<16, 1>(ft, g, e->stream, V, e->td, sb, 1, 1, R);
                    else launch_suffix<32, 1>(ft, g, e->stream, V, e->td, sb, 1, 1, R);
                }
                const int rc0 = check_launch(e);
                if (rc0) return rc0;
                /* the evaluation count: the lane kernel sums its own; after
                   the warp kernel, a thread per prefix (the pass is latency
                   bound) */
                if (!lanes) {
                    const unsigned cb = (unsigned)std::min<uint64_t>((R.count + 255) / 256,
                                                                     (uint64_t)e->sms * 32);
                    k_count_evals<<<std::max(cb, 1u), 256, 0, e->stream>>>(V, e->td, R, sb);
                }
            } else if (chunk == kLaneShape) {
                const int gl = e->grid(e->occ_mid_lanes);
                if (s == 2) {
                    if (t16) launch_mid_lanes<16, 2>(ft, gl, e->stream, V, e->td, sb, cpp, R);
                    else launch_mid_lanes<32, 2>(ft, gl, e->stream, V, e->td, sb, cpp, R);
                } else {
                    if (t16) launch_mid_lanes<16, 3>(ft, gl, e->stream, V, e->td, sb, cpp, R);
                    else launch_mid_lanes<32, 3>(ft, gl, e->stream, V, e->td, sb, cpp, R);
                }
            } else if (s == 2) {
                if (t16) launch_suffix<16, 2>(ft, g, e->stream, V, e->td, sb, cpp, chunk, R);
                else launch_suffix<32, 2>(ft, g, e->stream, V, e->td, sb, cpp, chunk, R);
            } else {
                if (t16) launch_suffix<16, 3>(ft, g, e->stream, V, e->td, sb, cpp, chunk, R);
                else launch_suffix<32, 3>(ft, g, e->stream, V, e->td, sb, cpp, chunk, R);
            }
            return check_launch(e);
        };
        tuned_ft = ft;
        tuned_ck = ck;
        /* task groups of the progressive mode: [first task, end task) with
           the level range they occupy */
        struct Group { int t0, t1; uint64_t b0, b1; };
        std::vector<Group> groups;
        if (!so && on_tasks && e->ntasks > 1) {
            const int nt = e->ntasks;
            const double per_group = 1.5 / std::max(e->t_eval_ms[s], 1e-12);
            int nact = 0;
            for (int t = 0; t < nt; t++) nact += e->h_active[t] ? 1 : 0;
            if (nact > 1) {
                uint64_t off = 0, gb0 = 0;
                int gt0 = 0;
                double acc = 0;
                for (int t = 0; t < nt; t++) {
                    uint64_t cnt = 0, ev = 0;
                    for (int m = 0; m < 128; m++) {
                        cnt += L.hist[(size_t)t * 128 + m];
                        ev += L.hist[(size_t)t * 128 + m] * gt.ev[s][m];
                    }
                    off += cnt;
                    if (e->h_active[t]) acc += (double)ev;
                    if (acc >= per_group || t == nt - 1) {
                        groups.push_back({gt0, t + 1, gb0, off});
                        gt0 = t + 1;
                        gb0 = off;
                        acc = 0;
                    }
                }
                if (off != L.n) groups.clear();   /* histogram and level disagree: one launch */
            }
        }
        if (groups.size() > 1) {
            for (const Group &G : groups) {
                if (G.b1 > G.b0) {
                    rc = launch(PrefixRange{nullptr, G.b0, G.b1 - G.b0});
                    if (rc) return rc;
                }
                CK(e_copy(e, &e->h_pin[kPinCount], e->d_small, 8, cudaMemcpyDeviceToHost,
                          e->stream));
                CK(cudaStreamSynchronize(e->stream));
                const uint64_t cnt = e->h_pin[kPinCount];
                if (cnt > taken) {
                    rc = take_records(e, S, K, runs, first_only, taken, cnt, 0);
                    if (rc) return rc;
                    taken = cnt;
                }
                (*on_tasks)(G.t0, G.t1);
            }
        } else {
            /* ordered stages start with `chunk` prefixes per launch and
               double it after every launch without a solution, so a stage
               that has to be searched completely takes O(log n) launches */
            uint64_t step = so && so->chunk ? so->chunk : std::max<uint64_t>(L.n, 1);
            for (uint64_t b0 = 0; b0 < L.n; b0 += step, step = so && so->chunk ? step * 2 : step) {
                const PrefixRange R{so ? so->order : nullptr, b0, std::min(step, L.n - b0)};
                rc = launch(R);
                if (rc) return rc;
                if (so && so->stop_at_first) {
                    const auto h0 = std::chrono::steady_clock::now();
                    CK(e_copy(e, &e->h_pin[kPinCount], e->d_small, 8, cudaMemcpyDeviceToHost,
                              e->stream));
                    cudaEventRecord(e->ev1, e->stream);
                    CK(cudaStreamSynchronize(e->stream));
                    /* the host side of a chunked launch: its wait beyond the
                       device work is what the next launch pays in idle time */
                    const double rt = std::chrono::duration<double, std::milli>(
                                          std::chrono::steady_clock::now() - h0).count();
                    if (e->measure) e->launch_rt_ms = 0.9 * e->launch_rt_ms + 0.1 * std::min(rt, 1.0);
                    if (e->h_pin[kPinCount]) {
                        so->prefixes_to_first = R.begin + R.count;
                        cudaEventElapsedTime(&so->ms_to_first, e->ev0, e->ev1);
                        stopped_early = R.begin + R.count < L.n;
                        break;
                    }
                }
            }
        }
    } else {
        set_err("suffix depth %d not supported (split too shallow)", s);
        return PCAGB_ENOMEM;
    }
    cudaEventRecord(e->ev1, e->stream);
    /* count, first key, (survivors), evaluations run so far in this solve */
    CK(e_copy(e, &e->h_pin[kPinCount], e->d_small, 32, cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    const unsigned long long nrec = e->h_pin[kPinCount], first = e->h_pin[kPinFirst];
    e->evals_run = e->h_pin[kPinCount + 3];
    float ms = 0;
    cudaEventElapsedTime(&ms, e->ev0, e->ev1);
    e->ms_suffix += ms;
    e->suffix_launches++;
    if (lane_launches == 1 && K < PCAGB_MAXD) {
        /* one launch: its events bracket it alone */
        float mk = 0;
        cudaEventElapsedTime(&mk, e->evk0, e->evk1);
        e->ms_lanes[K] += mk;
    }
    if (s >= 1 && !stopped_early && !(so && so->order) && e->measure) {
        /* value-class evaluations of this stage, for the autotuner */
        const std::vector<uint64_t> &g = gt.ev[s];
        uint64_t evals = 0;
        for (size_t i = 0; i < L.hist.size(); i++)
            if (e->h_active[i >> 7]) evals += L.hist[i] * g[i & 127];
        if (evals > 10000000ull) {
            const double per = ms / (double)evals;
            e->t_eval_ms[s] = 0.7 * e->t_eval_ms[s] + 0.3 * per;
            if (evals >= kTuneMinEvals && s <= 3 && nact_stage == 1) {
                if (tuned_ft >= 1) record_cost(e->ft_ms[s][tuned_ft], e->ft_n[s][tuned_ft], per);
                if (tuned_ck >= 0) record_cost(e->ck_ms[s][tuned_ck], e->ck_n[s][tuned_ck], per);
            }
        }
    }
    if (nrec <= taken) return PCAGB_OK;
    return take_records(e, S, K, runs, first_only, taken, nrec, first);
}

/* Host-side step for the reference-key dedup of the solving leaves
   (tools/enumerate.c:380-384 applies OEP to leaves too). */
void leaf_key(const task_spec_t *task, const search_state_t &root, const std::vector<uint16_t> &k,
              std::vector<uint8_t> *key)
{
    search_ctx_t ctx;
    search_ctx_init(&ctx, task);
    search_state_t s = root, n;
    for (uint16_t insn : k) {
        search_state_step(&ctx, &s, insn, &n);
        s = n;
    }
    key->clear();
    for (int t = 0; t < task->num_tests; t++) {
        const uint8_t *p = (const uint8_t *)s.regs[t];
        key->insert(key->end(), p, p + 16);
        key->push_back(s.flags[t]);
    }
}

/* Test order for the suffix kernel. Its lanes evaluate value classes on
   the first one or two tests and send survivors to a check of all tests, so
   the fewer classes pass the first tests the less work is done. The order is
   chosen greedily on (state, class) pairs sampled from the root and its
   children: each next test is the one the fewest remaining pairs pass. A
   permutation of the tests changes no result of the search (pruning keys,
   DFS order, programs and counts are all independent of it). */
std::vector<int> choose_test_order(const TaskRun &tr)
{
    const GenTables &gt = gen_tables();
    const int T = tr.T;
    search_ctx_t ctx;
    memset(&ctx, 0, sizeof ctx);
    ctx.num_tests = (uint8_t)T;
    /* the root and up to 24 of its children, spread over the op blocks */
    std::vector<search_state_t> sample(1, tr.root);
    uint16_t cands[4096];
    int n = gen_candidates(tr.root.live, cands, 4096);
    const int stride = std::max(1, n / 24);
    for (int i = 0; i < n; i += stride) {
        search_state_t c;
        if (search_state_step(&ctx, &tr.root, cands[i], &c)) sample.push_back(c);
    }
    std::vector<uint32_t> masks;
    for (const search_state_t &st : sample) {
        const uint32_t m = (st.live >> 1) & 127u;
        for (uint32_t i = gt.vc_off[m]; i < gt.vc_off[m + 1]; i++) {
            const uint32_t u = gt.vc_uop[i];
            uint32_t pass = 0;
            for (int t = 0; t < T; t++) {
                uint32_t v = pca_alu(UOP_OP(u), st.regs[t][UOP_A(u)], st.regs[t][UOP_B(u)],
                                     UOP_IMM(u));
                if (v == tr.target[t]) pass |= 1u << t;
            }
            masks.push_back(pass);
        }
    }
    std::vector<int> order;
    uint32_t used = 0;
    while ((int)order.size() < T && !masks.empty()) {
        int best = -1;
        size_t best_n = SIZE_MAX;
        for (int t = 0; t < T; t++) {
            if (used >> t & 1u) continue;
            size_t cnt = 0;
            for (uint32_t m : masks) cnt += m >> t & 1u;
            if (cnt < best_n) { best_n = cnt; best = t; }
        }
        order.push_back(best);
        used |= 1u << best;
        std::vector<uint32_t> keep;
        for (uint32_t m : masks)
            if (m >> best & 1u) keep.push_back(m);
        masks.swap(keep);
    }
    for (int t = 0; t < T; t++)
        if (!(used >> t & 1u)) order.push_back(t);
    return order;
}

uint64_t hist_sum(const Level &L, int t, const std::vector<uint64_t> &weight)
{
    uint64_t s = 0;
    for (int m = 0; m < 128; m++) s += L.hist[(size_t)t * 128 + m] * weight[m];
    return s;
}

/* Called once per task as soon as it is decided (proven optimal depth or
   depth limit reached), before the batch ends. */
typedef void (*done_fn)(int task, void *user);

/* Split-depth autotuner (first-only solves: the DFS-first optimal program
 * is the same whatever level the stage starts from, so the choice changes
 * the work, never the answer). The stage at depth K can start from any level S in
 * [K-3, K-1]; levels deeper than the ones built cost a build each (children
 * x measured ms per child + a fixed part), shrink the suffix work by the
 * measured dedup ratio, and are reused by later depths. The predicted
 * device time of each S is
 *   builds(D+1..S) + evals(S, K-S) x ms per evaluation,
 * with evals of a level not built yet extrapolated from the deepest built
 * level D: evals(S, K-S) ~ evals(D, K-D) x dedup_ratio^(S-D). The cheapest
 * S within the HBM budget (max_feasible) wins. stage_scale weights the
 * stage term (an ordered stage that stops at its first solution is expected
 * to run a fraction of it); *pred_ms receives the winner's predicted time.
 * With full_cap set, a level whose whole stage (builds + every prefix) is
 * predicted to cost more than full_cap is not chosen (-1 when none is
 * left). */
int autotune_split(pcagb_engine *e, int K, const std::vector<uint8_t> &active,
                   double stage_scale = 1.0, double *pred_ms = nullptr,
                   double full_cap = 1e300)
{
    const GenTables &gt = gen_tables();
    const int D = (int)e->levels.size() - 1;
    const int hi = std::min(K - 1, e->max_feasible);
    const int lo = std::max(0, K - 3);
    auto evals_from = [&](int S, int s) {
        const std::vector<uint64_t> &g = gt.ev[s];
        double ev = 0;
        const Level &L = e->levels[S];
        for (size_t i = 0; i < L.hist.size(); i++)
            if (active[i >> 7]) ev += (double)L.hist[i] * g[i & 127];
        return ev;
    };
    auto children_of = [&](int S) {
        double c = 0;
        const Level &L = e->levels[S];
        for (size_t i = 0; i < L.hist.size(); i++)
            if (active[i >> 7]) c += (double)L.hist[i] * gt.nc((int)(i & 127));
        return c;
    };
    if (hi <= D) {
        const int S = std::max(hi, lo);
        if (pred_ms)
            *pred_ms = K - S <= 3 && K - S >= 1
                           ? evals_from(S, K - S) * e->t_eval_ms[K - S] * stage_scale : 1e300;
        return S;
    }
    int best = -1;
    double best_ms = 1e300;
    for (int S = std::max(lo, 0); S <= hi; S++) {
        if (K - S > 3) continue;
        double ms, full;
        if (S <= D) {
            full = evals_from(S, K - S) * e->t_eval_ms[K - S];
            ms = full * stage_scale;
        } else {
            /* build D+1..S from D, then the suffix from S. A build that would
               not fit the arena (its table, bitmap and ranks, plus the new
               level sized at 1.5x the measured dedup ratio) is not chosen:
               it would only find that out after its insert. */
            double kids = children_of(D), build = 0, states_scale = 1.0;
            double parents = (double)e->levels[D].n, held = 0;
            const double state_bytes = 16.0 * e->TPC + e->TPC + 12 + 64;
            const double free_b = (double)(e->top - e->bottom);
            bool fits = true;
            for (int d = D + 1; d <= S; d++) {
                /* the last stage's split level is built lean */
                const bool lean = d == S && S == K - 1 && K == e->lean_K;
                build += kids * (lean ? e->t_child_lean_ms : e->t_child_ms) + e->t_build_fixed_ms;
                double slots = 1024;
                while (slots < 2 * kids) slots *= 2;
                const double states = kids * std::min(1.0, 1.5 * e->dedup_ratio);
                held += (parents + 1) * 8 + states * state_bytes;
                if (held + slots * 8 + kids / 32 * 12 > free_b) fits = false;
                states_scale *= e->dedup_ratio;
                parents = kids * e->dedup_ratio;
                kids *= e->dedup_ratio * 800.0;  /* ~children per state deeper down */
            }
            if (!fits) continue;
            const double stage = evals_from(D, K - D) * states_scale * e->t_eval_ms[K - S];
            full = build + stage;
            ms = build + stage * stage_scale;
        }
        if (full > full_cap) continue;
        if (ms < best_ms) { best_ms = ms; best = S; }
    }
    if (pred_ms) *pred_ms = best_ms;
    if (best < 0) return full_cap < 1e300 ? -1 : std::max(hi, lo);
    return best;
}

typedef CUresult (*AddressRangeFn)(CUdeviceptr *, size_t *, CUdeviceptr);

AddressRangeFn address_range_fn()
{
    static AddressRangeFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuMemGetAddressRange", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (AddressRangeFn)p;
    });
    return fn;
}

/* An order callback's array must be device memory of this engine's GPU
 * holding n uint32 values that form a permutation of 0..n-1: anything else
 * would skip prefixes (a depth left unproven) or index outside the level. */
int validate_order(pcagb_engine *e, const uint32_t *order, uint64_t n)
{
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, order) != cudaSuccess ||
        (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged) ||
        a.device != e->device) {
        cudaGetLastError();
        set_err("order callback returned %p: not device memory of GPU %d", (const void *)order,
                e->device);
        return PCAGB_EINVAL;
    }
    if (AddressRangeFn fn = address_range_fn()) {
        CUdeviceptr base = 0;
        size_t size = 0;
        const CUdeviceptr p = (CUdeviceptr)(uintptr_t)order;
        if (fn(&base, &size, p) != CUDA_SUCCESS || p + n * sizeof(uint32_t) > base + size) {
            set_err("order callback returned an array shorter than the level (%llu prefixes)",
                    (unsigned long long)n);
            return PCAGB_EINVAL;
        }
    }
    const size_t saved = e->top;
    unsigned long long *bad = (unsigned long long *)e->alloc_top(sizeof(unsigned long long));
    uint32_t *seen = (uint32_t *)e->alloc_top(((n + 31) / 32) * sizeof(uint32_t));
    if (!bad || !seen) {
        e->top = saved;
        set_err("arena exhausted checking an order");
        return PCAGB_ENOMEM;
    }
    CK(cudaMemsetAsync(bad, 0, sizeof *bad, e->stream));
    CK(cudaMemsetAsync(seen, 0, ((n + 31) / 32) * sizeof(uint32_t), e->stream));
    k_check_perm<<<e->grid(4), 256, 0, e->stream>>>(order, n, seen, bad);
    int rc = check_launch(e);
    unsigned long long nbad = 0;
    if (!rc) {
        CK(e_copy(e, &nbad, bad, sizeof nbad, cudaMemcpyDeviceToHost, e->stream));
        CK(cudaStreamSynchronize(e->stream));
    }
    e->top = saved;
    if (rc) return rc;
    if (nbad) {
        set_err("order callback returned no permutation of the %llu prefixes (%llu bad entries)",
                (unsigned long long)n, nbad);
        return PCAGB_EINVAL;
    }
    return PCAGB_OK;
}

/* Core batched IDDFS shared by every solve entry point. */
struct OrderSpec {
    pcagb_order_cb cb = nullptr;
    void *user = nullptr;
    uint64_t chunk = 0;
};

int run_batch(pcagb_engine *e, std::vector<TaskRun> &runs, const pcagb_opts_t &o,
              done_fn on_done = nullptr, void *user = nullptr, const OrderSpec *ord = nullptr)
{
    const GenTables &gt = gen_tables();
    auto t_start = std::chrono::steady_clock::now();
    auto elapsed = [&] {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    };
    const int nt = (int)runs.size();
    if (nt < 1 || nt > kMaxBatch) {
        set_err("batch of %d tasks (1..%d)", nt, kMaxBatch);
        return PCAGB_EINVAL;
    }
    e->ntasks = nt;
    e->levels.clear();
    e->bottom = 0;
    e->top = e->cap;
    e->ms_expand = e->ms_suffix = e->ms_insert = 0;
    std::fill(e->ms_lanes, e->ms_lanes + PCAGB_MAXD, 0.0);
    e->launches = 0;
    e->h2d = e->d2h = 0;
    e->insert_launches = e->suffix_launches = e->insert_children = 0;
    e->evals_run = 0;
    e->force_ft = o.first_tests;
    e->force_chunk = o.suffix_chunk;
    e->measure = o.shared_gpu == 0;
    /* a shared solve takes the costs its device's unshared solves measured */
    if (!e->measure) load_costs(e);
    e->max_feasible = SEARCH_MAX_DEPTH;
    int maxT = 0, maxK = 0;
    for (TaskRun &tr : runs) {
        maxT = std::max(maxT, tr.T);
        maxK = std::max(maxK, tr.max_depth);
        memset(&tr.res, 0, sizeof tr.res);
        tr.res.optimal_depth = -1;
        tr.order = choose_test_order(tr);
    }
    e->TPC = maxT <= 16 ? 16 : 32;
    e->no_oep = o.oep_mode == PCAGB_OEP_NONE;
    /* the last depth's split level may be built lean when nothing but its
       lane-per-prefix stage reads it: not for the reference's counters (every
       level to K), an ordered solve (its callback sees the level), a forced
       warp per prefix at depth 1, or a caller that asks for full levels */
    const bool warp_forced = o.suffix_chunk >= 1 && o.suffix_chunk < 32;
    e->lean_K = !o.count_levels && !ord && !warp_forced && !o.full_levels ? maxK : -1;
    e->td = TaskDev{e->d_task_T, e->d_task_target, e->d_task_active,
                    o.oep_mode == PCAGB_OEP_EXACT_LIVE, o.oep_mode != PCAGB_OEP_NONE};
    CK(cudaSetDevice(e->device));
    CK(cudaMemsetAsync(e->d_status, 0, 4, e->stream));
    CK(cudaMemsetAsync(e->d_small + 3, 0, 8, e->stream));
    {
        std::vector<int32_t> T(nt);
        std::vector<uint32_t> tgt((size_t)nt * 32, 0);
        for (int i = 0; i < nt; i++) {
            T[i] = runs[i].T;
            for (int t = 0; t < runs[i].T; t++)
                tgt[(size_t)i * 32 + t] = runs[i].target[runs[i].order[t]];
        }
        std::vector<uint16_t> io((size_t)nt * 3 * 32, 0);
        for (int i = 0; i < nt; i++)
            for (int t = 0; t < runs[i].T; t++) {
                const int o = runs[i].order[t];
                io[((size_t)i * 3 + 0) * 32 + t] = runs[i].root.regs[o][1];
                io[((size_t)i * 3 + 1) * 32 + t] = runs[i].root.regs[o][2];
                io[((size_t)i * 3 + 2) * 32 + t] = runs[i].target[o];
            }
        CK(e_copy(e, e->d_task_T, T.data(), nt * 4, cudaMemcpyHostToDevice, e->stream));
        CK(e_copy(e, e->d_task_target, tgt.data(), tgt.size() * 4, cudaMemcpyHostToDevice,
                  e->stream));
        CK(e_copy(e, e->d_task_io, io.data(), io.size() * 2, cudaMemcpyHostToDevice, e->stream));
    }

    /* level 0: one root per task */
    Level L0;
    if (alloc_level(e, L0, nt) != PCAGB_OK) { set_err("arena too small"); return PCAGB_ENOMEM; }
    {
        const int TPC = e->TPC;
        std::vector<uint16_t> regs((size_t)nt * 8 * TPC, 0), probe((size_t)nt * 32, 0);
        std::vector<uint8_t> flags((size_t)nt * TPC, 0), live(nt);
        std::vector<uint16_t> task(nt), cidx(nt, 0);
        std::vector<uint32_t> parent(nt, 0);
        L0.hist.assign((size_t)nt * 128, 0);
        for (int i = 0; i < nt; i++) {
            const TaskRun &tr = runs[i];
            for (int t = 0; t < tr.T; t++) {
                for (int r = 1; r < 8; r++) {
                    regs[((size_t)i * 8 + r) * TPC + t] = tr.root.regs[tr.order[t]][r];
                    if (t < 4) probe[(size_t)i * 32 + r * 4 + t] = tr.root.regs[tr.order[t]][r];
                }
                flags[(size_t)i * TPC + t] = tr.root.flags[tr.order[t]];
            }
            live[i] = tr.root.live;
            task[i] = (uint16_t)i;
            L0.hist[(size_t)i * 128 + ((tr.root.live >> 1) & 127)] = 1;
        }
        CK(e_copy(e, L0.regs, regs.data(), regs.size() * 2, cudaMemcpyHostToDevice, e->stream));
        CK(e_copy(e, L0.flags, flags.data(), flags.size(), cudaMemcpyHostToDevice, e->stream));
        CK(e_copy(e, L0.live, live.data(), nt, cudaMemcpyHostToDevice, e->stream));
        CK(e_copy(e, L0.task, task.data(), nt * 2, cudaMemcpyHostToDevice, e->stream));
        CK(e_copy(e, L0.parent, parent.data(), nt * 4, cudaMemcpyHostToDevice, e->stream));
        CK(e_copy(e, L0.cidx, cidx.data(), nt * 2, cudaMemcpyHostToDevice, e->stream));
        CK(cudaMemsetAsync(L0.rdl, 0, nt, e->stream));
        CK(cudaMemsetAsync(L0.own, 0, nt, e->stream));
        CK(cudaMemsetAsync(L0.twin, 0, nt, e->stream));
        CK(e_copy(e, L0.probe, probe.data(), probe.size() * 2, cudaMemcpyHostToDevice, e->stream));
    }
    e->levels.push_back(std::move(L0));

    /* K = 0: does a live register already hold the target? */
    for (TaskRun &tr : runs) {
        tr.res.level_children[0] = tr.res.level_survivors[0] = 1;
        if (tr.min_depth > 0) continue;
        for (uint32_t r = 1; r < 8; r++) {
            if (!((tr.root.live >> r) & 1u)) continue;
            bool ok = true;
            for (int t = 0; t < tr.T && ok; t++) ok = tr.root.regs[t][r] == tr.target[t];
            if (ok) {
                RawSol s0;
                s0.out_reg = r;
                s0.key.push_back(r);
                tr.sols.push_back(s0);
            }
        }
        if (!tr.sols.empty()) {
            tr.done = true;
            tr.optimal_depth = 0;
            tr.res.tried[0] = tr.sols.size();
            tr.t_done = elapsed();
        }
    }
    std::vector<uint8_t> notified(nt, 0);
    auto notify = [&](int i) {
        if (notified[i]) return;
        notified[i] = 1;
        TaskRun &tr = runs[i];
        tr.res.optimal_depth = tr.optimal_depth;
        tr.res.seconds = tr.t_done;
        if (on_done) on_done(i, user);
    };
    for (int i = 0; i < nt; i++)
        if (runs[i].done) notify(i);
    std::vector<uint8_t> active(nt, 0);
    std::vector<uint64_t> pruned_cum(nt, 0);
    std::vector<uint64_t> nc_w(128), ones(128, 1);
    for (int m = 0; m < 128; m++) nc_w[m] = gt.nc(m);
    for (int K = 1; K <= maxK; K++) {
        int nact = 0;
        for (int i = 0; i < nt; i++) {
            TaskRun &tr = runs[i];
            if (!tr.done && K > tr.max_depth) {
                tr.done = true;
                tr.t_done = elapsed();
                notify(i);
            }
            active[i] = !tr.done;
            nact += active[i];
        }
        if (!nact) break;
        CK(e_copy(e, e->d_task_active, active.data(), nt, cudaMemcpyHostToDevice, e->stream));
        e->h_active = active;
        int S_target = o.count_levels ? K : K - 1;
        /* an ordered solve with an automatic split orders only the stages
           worth it: a stage the autotuner expects to finish in under
           kOrderMinStageMs runs plain from its cheapest level; the others
           start from the level that minimises builds + a tenth of the stage
           (the share an ordered stage is expected to run) among the levels
           whose whole stage is predicted within kOrderMaxOverhead of the
           plain choice's: a depth without a solution is searched completely
           in any order, and then costs about what the plain solve pays */
        bool ordered_stage = ord != nullptr;
        if (o.split_depth >= 0) {
            S_target = std::min(S_target, o.split_depth);
        } else if (ord && !o.count_levels) {
            double plain_ms = 0;
            const int Sp = autotune_split(e, K, active, 1.0, &plain_ms);
            if (plain_ms < kOrderMinStageMs) {
                S_target = Sp;
                ordered_stage = false;
            } else {
                const int So = autotune_split(e, K, active, kOrderStageShare, nullptr,
                                              plain_ms * kOrderMaxOverhead);
                S_target = So >= 0 ? So : Sp;
            }
        } else if (o.first_only && !o.count_levels) {
            S_target = autotune_split(e, K, active);
        }
        while ((int)e->levels.size() - 1 < S_target &&
               (int)e->levels.size() - 1 < e->max_feasible) {
            const int d = (int)e->levels.size() - 1;
            /* the last depth's split level, read by nothing but its
               last-position stage, is built lean */
            const bool lean = K == e->lean_K && d + 1 == S_target && S_target == K - 1;
            int rc = build_level(e, d, lean);
            if (rc == PCAGB_ENOMEM) {
                e->max_feasible = d;
                break;
            }
            if (rc) return rc;
        }
        const int S = std::min(S_target, (int)e->levels.size() - 1);
        const int s = K - S;
        if (o.count_levels && S < S_target) {
            set_err("count_levels: level %d does not fit the HBM budget", S + 1);
            return PCAGB_ENOMEM;
        }
        if (s > 3) {
            set_err("depth %d needs level %d in HBM; the budget holds level %d", K, K - 3, S);
            return PCAGB_ENOMEM;
        }
        /* evaluations: value classes scanned at the last position */
        const std::vector<uint64_t> &g = gt.ev[std::max(s, 1)];
        const Level &LS = e->levels[S];
        for (int i = 0; i < nt; i++) {
            if (!active[i]) continue;
            TaskRun &tr = runs[i];
            tr.res.split_used = S;
            tr.res.candidates[K] = s == 0 ? hist_sum(LS, i, ones) : hist_sum(LS, i, gt.f[s]);
            tr.res.evaluations[K] = s == 0 ? tr.res.candidates[K] : hist_sum(LS, i, g);
            for (int d = 1; d <= S; d++) {
                tr.res.level_children[d] = hist_sum(e->levels[d - 1], i, nc_w);
                tr.res.level_survivors[d] = hist_sum(e->levels[d], i, ones);
            }
            tr.nrec = 0;
        }
        StageOrder so;
        StageOrder *sop = nullptr;
        if (ordered_stage && s >= 1) {
            double evals = 0;
            for (int i = 0; i < nt; i++)
                if (active[i]) evals += (double)runs[i].res.evaluations[K];
            pcagb_level_view_t lv{LS.regs, LS.flags, LS.live, LS.task, LS.n, e->TPC, S, K, nt,
                                  e->d_task_io, e->d_task_T, (void *)e->stream,
                                  evals * e->t_eval_ms[s]};
            so.order = ord->cb ? ord->cb(&lv, ord->user) : nullptr;
            if (so.order) {
                const int vrc = validate_order(e, so.order, LS.n);
                if (vrc) return vrc;
            }
            so.chunk = ord->chunk;
            so.stop_at_first = true;
            sop = &so;
        } else if (s >= 1 && nt == 1 && o.first_only && !o.count_levels && !ord &&
                   o.stage_launch >= 0) {
            /* a first-only stage of one task in chunks of DFS order, stopping
               at the first launch that holds a solution (every earlier
               prefix is searched, so its solutions hold the DFS-first one):
               worth it when the stage is predicted to take much longer than
               the host round trip each launch adds */
            uint64_t c0 = o.stage_launch > 0 ? (uint64_t)o.stage_launch : 0;
            if (!c0) {
                double evals = 0;
                for (int i = 0; i < nt; i++)
                    if (active[i]) evals += (double)runs[i].res.evaluations[K];
                if (evals * e->t_eval_ms[s] > 32.0 * e->launch_rt_ms && LS.n >= 256)
                    c0 = std::max<uint64_t>(LS.n / 16, 1);
            }
            if (c0) {
                so.order = nullptr;
                so.chunk = c0;
                so.stop_at_first = true;
                sop = &so;
            }
        }
        /* a task searched at depth K: its counters, and done when it has
           solutions or K is its last depth */
        std::vector<uint8_t> finished(nt, 0);
        auto finish = [&](int i) {
            if (!active[i] || finished[i]) return;
            finished[i] = 1;
            TaskRun &tr = runs[i];
            /* the reference's counters (exact when every level up to K is built) */
            uint64_t tried = 0, pruned = 0;
            for (int j = 1; j <= S; j++) {
                tried += tr.res.level_children[j];
                pruned += tr.res.level_children[j] - tr.res.level_survivors[j];
            }
            for (int k = 1; k <= s; k++) tried += hist_sum(LS, i, gt.f[k]);
            pruned_cum[i] += pruned;
            tr.res.tried[K] = tried + (s == 0 ? tr.nrec : 0);
            tr.res.pruned_cum[K] = pruned_cum[i];
            if (tr.nrec) {
                tr.done = true;
                tr.optimal_depth = K;
                tr.t_done = elapsed();
                tr.res.prefixes_at_optimal = LS.n;
                tr.res.prefixes_to_first = sop ? sop->prefixes_to_first : LS.n;
                tr.res.ms_to_first = sop ? sop->ms_to_first : 0.0;
                tr.res.total_solutions =
                    s == 0 || (o.first_only && nt == 1) ? tr.nrec : tr.sols.size();
                notify(i);
            } else if (K >= tr.max_depth) {
                tr.done = true;
                tr.t_done = elapsed();
                notify(i);
            }
        };
        const std::function<void(int, int)> on_tasks = [&](int lo, int hi) {
            for (int i = lo; i < hi; i++) finish(i);
        };
        /* a plain stage of an ordered solve keeps only the DFS-first
           solution, as a first-only solve does */
        const bool stage_first_only = o.first_only != 0 || (ord && !ordered_stage);
        int rc = run_stage(e, S, K, runs, stage_first_only, sop, sop ? nullptr : &on_tasks);
        if (rc) return rc;
        for (int i = 0; i < nt; i++) finish(i);
    }
    const double total = elapsed();
    for (TaskRun &tr : runs) {
        if (!tr.done) tr.t_done = total;
        tr.res.optimal_depth = tr.optimal_depth;
        if (tr.optimal_depth == 0) tr.res.total_solutions = tr.sols.size();
        tr.res.gpu_ms_expand = e->ms_expand;
        tr.res.gpu_ms_suffix = e->ms_suffix;
        tr.res.gpu_ms_insert = e->ms_insert;
        tr.res.kernel_launches = e->launches;
        tr.res.insert_launches = e->insert_launches;
        tr.res.suffix_launches = e->suffix_launches;
        tr.res.insert_children = e->insert_children;
        tr.res.evaluations_run = e->evals_run;
        std::copy(e->ms_lanes, e->ms_lanes + PCAGB_MAXD, tr.res.gpu_ms_lanes);
        tr.res.h2d_bytes = e->h2d;
        tr.res.d2h_bytes = e->d2h;
        tr.res.seconds = tr.t_done;
    }
    for (int i = 0; i < nt; i++) notify(i);
    if (e->measure) store_costs(e);
    return PCAGB_OK;
}

/* The candidate tables are the same for every engine on a device, and the
   kernels reach them through __constant__ symbols shared by the whole
   device. They are uploaded once per device and live until the process
   exits, so destroying one engine never leaves another engine's kernels
   reading freed memory. */
std::mutex g_tables_mu;
bool g_tables_ready[64];

int ensure_device_tables(int device)
{
    std::lock_guard<std::mutex> lk(g_tables_mu);
    if (device < 0 || device >= 64) { set_err("device %d out of range", device); return PCAGB_EINVAL; }
    if (g_tables_ready[device]) return PCAGB_OK;
    const GenTables &gt = gen_tables();
    std::vector<uint16_t> first(gt.vc_uop.size(), 0);
    for (int m = 0; m < 128; m++) {
        std::vector<bool> seen(gt.nvc(m), false);
        for (uint32_t c = 0; c < (uint32_t)gt.nc(m); c++) {
            uint16_t v = gt.cand_vc[gt.cand_off[m] + c];
            if (!seen[v]) { seen[v] = true; first[gt.vc_off[m] + v] = (uint16_t)c; }
        }
    }
    uint32_t *cand_uop = nullptr, *vc_uop = nullptr, *chunks = nullptr, *vcr_uop_d = nullptr;
    uint16_t *vc_first = nullptr, *vcr = nullptr;
    {
        std::vector<uint32_t> vcr_uop(gt.vcr.size());
        for (int m = 0; m < 128; m++)
            for (uint32_t k = gt.vcr_off[m * 8]; k < gt.vcr_off[m * 8 + 8]; k++)
                vcr_uop[k] = gt.vc_uop[gt.vc_off[m] + gt.vcr[k]];
        CK(cudaMalloc(&vcr_uop_d, std::max<size_t>(vcr_uop.size(), 1) * 4));
        CK(cudaMalloc(&vcr, std::max<size_t>(gt.vcr.size(), 1) * 2));
        CK(cudaMemcpy(vcr_uop_d, vcr_uop.data(), vcr_uop.size() * 4, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(vcr, gt.vcr.data(), gt.vcr.size() * 2, cudaMemcpyHostToDevice));
        const uint32_t *vu = vcr_uop_d;
        const uint16_t *vr = vcr;
        CK(cudaMemcpyToSymbol(c_vcr_off, gt.vcr_off.data(), gt.vcr_off.size() * 4));
        CK(cudaMemcpyToSymbol(c_vcr_uop, &vu, sizeof vu));
        CK(cudaMemcpyToSymbol(c_vcr, &vr, sizeof vr));
    }
    {
        uint32_t *pr = nullptr;
        uint16_t *pr_cls = nullptr;
        CK(cudaMalloc(&pr, std::max<size_t>(gt.pr.size(), 1) * 4));
        CK(cudaMalloc(&pr_cls, std::max<size_t>(gt.pr_cls.size(), 1) * 2));
        CK(cudaMemcpy(pr, gt.pr.data(), gt.pr.size() * 4, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(pr_cls, gt.pr_cls.data(), gt.pr_cls.size() * 2, cudaMemcpyHostToDevice));
        const uint32_t *pp = pr;
        const uint16_t *pc = pr_cls;
        CK(cudaMemcpyToSymbol(c_pr_off, gt.pr_off.data(), gt.pr_off.size() * 4));
        CK(cudaMemcpyToSymbol(c_pr_ev, gt.pr_ev.data(), gt.pr_ev.size() * 4));
        /* the same counts in global memory for k_count_evals, whose lanes
           read different entries (constant memory serialises those); entry
           (m, 0) is a root's scan: every class of mask m */
        std::vector<uint32_t> ev1(128 * 8);
        for (int m = 0; m < 128; m++)
            for (int r = 0; r < 8; r++)
                ev1[m * 8 + r] = r ? gt.pr_ev[m * 8 + r] : (uint32_t)gt.nvc(m);
        uint32_t *ev1_d = nullptr;
        CK(cudaMalloc(&ev1_d, ev1.size() * 4));
        CK(cudaMemcpy(ev1_d, ev1.data(), ev1.size() * 4, cudaMemcpyHostToDevice));
        const uint32_t *ev1p = ev1_d;
        CK(cudaMemcpyToSymbol(c_ev_sd1, &ev1p, sizeof ev1p));
        uint32_t *pro_d = nullptr;
        CK(cudaMalloc(&pro_d, gt.pr_off.size() * 4));
        CK(cudaMemcpy(pro_d, gt.pr_off.data(), gt.pr_off.size() * 4, cudaMemcpyHostToDevice));
        const uint32_t *prop = pro_d;
        CK(cudaMemcpyToSymbol(c_pr_off_g, &prop, sizeof prop));
        CK(cudaMemcpyToSymbol(c_pr, &pp, sizeof pp));
        CK(cudaMemcpyToSymbol(c_pr_cls, &pc, sizeof pc));
    }
    CK(cudaMalloc(&cand_uop, gt.cand_uop.size() * 4));
    CK(cudaMalloc(&vc_uop, gt.vc_uop.size() * 4));
    CK(cudaMalloc(&vc_first, first.size() * 2));
    CK(cudaMalloc(&chunks, gt.chunks.size() * 4));
    {
        /* bit 31 of a device micro-op marks a candidate whose child is an
           earlier sibling's state (cand_dupe); the field macros ignore it */
        std::vector<uint32_t> cu_flagged(gt.cand_uop);
        for (size_t i = 0; i < cu_flagged.size(); i++)
            if (gt.cand_dupe[i]) cu_flagged[i] |= 1u << 31;
        CK(cudaMemcpy(cand_uop, cu_flagged.data(), cu_flagged.size() * 4, cudaMemcpyHostToDevice));
    }
    CK(cudaMemcpy(vc_uop, gt.vc_uop.data(), gt.vc_uop.size() * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(vc_first, first.data(), first.size() * 2, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(chunks, gt.chunks.data(), gt.chunks.size() * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpyToSymbol(c_cand_off, gt.cand_off.data(), 129 * 4));
    CK(cudaMemcpyToSymbol(c_vc_off, gt.vc_off.data(), 129 * 4));
    CK(cudaMemcpyToSymbol(c_chunk_off, gt.chunk_off.data(), 129 * 4));
    const uint32_t *cu = cand_uop, *vu = vc_uop, *ck = chunks;
    const uint16_t *vf = vc_first;
    CK(cudaMemcpyToSymbol(c_cand_uop, &cu, sizeof cu));
    CK(cudaMemcpyToSymbol(c_vc_uop, &vu, sizeof vu));
    CK(cudaMemcpyToSymbol(c_vc_first, &vf, sizeof vf));
    CK(cudaMemcpyToSymbol(c_chunks, &ck, sizeof ck));
    CK(cudaDeviceSynchronize());
    g_tables_ready[device] = true;
    return PCAGB_OK;
}

int engine_init(pcagb_engine *e, int device, size_t budget)
{
    CK(cudaSetDevice(device));
    e->device = device;
    load_costs(e);
    CK(cudaDeviceGetAttribute(&e->sms, cudaDevAttrMultiProcessorCount, device));
    CK(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
    CK(cudaEventCreate(&e->ev0));
    CK(cudaEventCreate(&e->ev1));
    CK(cudaEventCreate(&e->ev2));
    CK(cudaEventCreate(&e->ev3));
    CK(cudaEventCreate(&e->evk0));
    CK(cudaEventCreate(&e->evk1));
    {
        /* CUDA loads a kernel at its first launch; load them all now, so no
           solve pays a module load inside its timing (the autotuner's
           measured costs) or a served request's latency */
        cudaFuncAttributes fa;
#define PCAGB_PRELOAD(...) cudaFuncGetAttributes(&fa, __VA_ARGS__)
        PCAGB_PRELOAD(k_suffix<16, 1, 1>); PCAGB_PRELOAD(k_suffix<16, 1, 2>);
        PCAGB_PRELOAD(k_suffix<16, 1, 3>); PCAGB_PRELOAD(k_suffix<16, 2, 1>);
        PCAGB_PRELOAD(k_suffix<16, 2, 2>); PCAGB_PRELOAD(k_suffix<16, 2, 3>);
        PCAGB_PRELOAD(k_suffix<16, 3, 1>); PCAGB_PRELOAD(k_suffix<16, 3, 2>);
        PCAGB_PRELOAD(k_suffix<16, 3, 3>); PCAGB_PRELOAD(k_suffix<32, 1, 1>);
        PCAGB_PRELOAD(k_suffix<32, 1, 2>); PCAGB_PRELOAD(k_suffix<32, 1, 3>);
        PCAGB_PRELOAD(k_suffix<32, 2, 1>); PCAGB_PRELOAD(k_suffix<32, 2, 2>);
        PCAGB_PRELOAD(k_suffix<32, 2, 3>); PCAGB_PRELOAD(k_suffix<32, 3, 1>);
        PCAGB_PRELOAD(k_suffix<32, 3, 2>); PCAGB_PRELOAD(k_suffix<32, 3, 3>);
        PCAGB_PRELOAD(k_suffix_lanes<16, 1>); PCAGB_PRELOAD(k_suffix_lanes<16, 2>);
        PCAGB_PRELOAD(k_suffix_lanes<16, 3>); PCAGB_PRELOAD(k_suffix_lanes<32, 1>);
        PCAGB_PRELOAD(k_suffix_lanes<32, 2>); PCAGB_PRELOAD(k_suffix_lanes<32, 3>);
        PCAGB_PRELOAD(k_suffix_mid_lanes<16, 2, 1>); PCAGB_PRELOAD(k_suffix_mid_lanes<16, 2, 2>);
        PCAGB_PRELOAD(k_suffix_mid_lanes<16, 2, 3>); PCAGB_PRELOAD(k_suffix_mid_lanes<16, 3, 1>);
        PCAGB_PRELOAD(k_suffix_mid_lanes<16, 3, 2>); PCAGB_PRELOAD(k_suffix_mid_lanes<16, 3, 3>);
        PCAGB_PRELOAD(k_suffix_mid_lanes<32, 2, 1>); PCAGB_PRELOAD(k_suffix_mid_lanes<32, 2, 2>);
        PCAGB_PRELOAD(k_suffix_mid_lanes<32, 2, 3>); PCAGB_PRELOAD(k_suffix_mid_lanes<32, 3, 1>);
        PCAGB_PRELOAD(k_suffix_mid_lanes<32, 3, 2>); PCAGB_PRELOAD(k_suffix_mid_lanes<32, 3, 3>);
        PCAGB_PRELOAD(k_expand_insert<16>); PCAGB_PRELOAD(k_expand_insert<32>);
        PCAGB_PRELOAD(k_materialize<16>); PCAGB_PRELOAD(k_materialize<32>);
        PCAGB_PRELOAD(k_twins<16>); PCAGB_PRELOAD(k_twins<32>);
        PCAGB_PRELOAD(k_leaf<16>); PCAGB_PRELOAD(k_leaf<32>);
        PCAGB_PRELOAD(k_count_evals); PCAGB_PRELOAD(k_mark); PCAGB_PRELOAD(k_mark_all);
        PCAGB_PRELOAD(k_popc); PCAGB_PRELOAD(k_child_counts); PCAGB_PRELOAD(k_task_hist);
        PCAGB_PRELOAD(k_task_hist_smem); PCAGB_PRELOAD(k_scan_local); PCAGB_PRELOAD(k_scan_add);
        PCAGB_PRELOAD(k_gather_paths); PCAGB_PRELOAD(k_check_perm);
#undef PCAGB_PRELOAD
        cudaGetLastError();
        /* the insert kernel keeps each warp's children in shared memory:
           its occupancy needs the largest shared-memory carveout */
        cudaFuncSetAttribute(k_expand_insert<32>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
        cudaFuncSetAttribute(k_expand_insert<16>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
        int nb = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_expand_insert<32>, kThreads, 0) ==
                cudaSuccess && nb > 0)
            e->occ_insert = nb;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_suffix<32, 1, 2>, kThreads, 0) ==
                cudaSuccess && nb > 0)
            e->occ_suffix = nb;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_materialize<32>, kThreads, 0) ==
                cudaSuccess && nb > 0)
            e->occ_mat = nb;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_suffix_lanes<32, 2>, kThreads, 0) ==
                cudaSuccess && nb > 0)
            e->occ_lanes = nb;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_suffix_mid_lanes<32, 2, 2>,
                                                          kThreads, 0) == cudaSuccess && nb > 0)
            e->occ_mid_lanes = nb;
        cudaGetLastError();
    }
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    if (budget == kArenaExternal) {
        /* the arena comes with each solve (pcagb_internal_solve_batch_arena) */
        e->arena = nullptr;
        e->cap = e->top = 0;
    } else {
        if (budget == 0) budget = (size_t)(free_b * 0.6);
        if (budget > free_b) budget = free_b - (256u << 20);
        budget &= ~size_t(4095);
        CK(cudaMalloc(&e->arena, budget));
        e->cap = budget;
        e->top = budget;
    }
    int trc = ensure_device_tables(device);
    if (trc) return trc;
    CK(cudaMalloc(&e->d_small, 256 * sizeof(unsigned long long)));
    CK(cudaMalloc(&e->d_status, 16));
    CK(cudaMalloc(&e->d_sol, e->sol_cap * sizeof(ulonglong2)));
    CK(cudaMalloc(&e->d_task_T, kMaxBatch * 4));
    CK(cudaMalloc(&e->d_task_target, (size_t)kMaxBatch * 32 * 4));
    CK(cudaMalloc(&e->d_task_active, kMaxBatch));
    CK(cudaMalloc(&e->d_task_io, (size_t)kMaxBatch * 3 * 32 * 2));
    CK(cudaMalloc(&e->d_hist, (size_t)kMaxBatch * 128 * sizeof(unsigned long long)));
    CK(cudaMallocHost(&e->h_pin, (kPinHist + (size_t)kMaxBatch * 128) * sizeof(unsigned long long)));
    return PCAGB_OK;
}

bool make_run(const task_spec_t *task, const pcagb_opts_t &o, TaskRun *tr)
{
    search_ctx_t ctx;
    if (search_ctx_init(&ctx, task) != 0 || task->num_tests < 1) {
        set_err("task needs 1..32 tests, one output and at most 7 inputs");
        return false;
    }
    if (o.max_depth < 0 || o.max_depth > 12 || task->num_inputs + o.max_depth + 2 > 16) {
        set_err("max_depth %d out of range (program length is limited to 16)", o.max_depth);
        return false;
    }
    if (o.first_tests < 0 || o.first_tests > 3 || o.suffix_chunk < 0 ||
        (o.suffix_chunk > 64 && o.suffix_chunk != (int)kLaneShape) ||
        o.stage_launch < -1) {
        set_err("launch choices out of range (first_tests 0..3, suffix_chunk 0..64 or 1024, "
                "stage_launch >= -1)");
        return false;
    }
    search_state_init_root(&ctx, &tr->root);
    tr->T = task->num_tests;
    for (int t = 0; t < tr->T; t++) tr->target[t] = task->tests[t].out[0];
    tr->max_depth = o.max_depth;
    tr->min_depth = o.min_depth;
    return true;
}

/* Write a task's solutions (full programs, VM re-checked) to the caller. */
int emit_solutions(const task_spec_t *task, const pcagb_opts_t &o, TaskRun &tr,
                   uint16_t *sol_progs, int *sol_lens, int sol_cap)
{
    std::vector<RawSol> &sols = tr.sols;
    /* The reference applies its pruner to the last level too: among solving
       programs with equal final regs+flags only the DFS-first is printed. */
    if (o.oep_mode == PCAGB_OEP_EXACT && !o.count_levels && tr.optimal_depth > 0 &&
        !o.first_only) {
        std::vector<RawSol> kept;
        std::vector<std::vector<uint8_t>> seen;
        std::vector<uint8_t> key;
        for (RawSol &s : sols) {
            leaf_key(task, tr.root, s.kernel, &key);
            if (std::find(seen.begin(), seen.end(), key) != seen.end()) continue;
            seen.push_back(key);
            kept.push_back(s);
        }
        sols.swap(kept);
        tr.res.total_solutions = sols.size();
    }
    int stored = 0;
    for (const RawSol &s : sols) {
        if (stored >= sol_cap || !sol_progs || (o.first_only && stored == 1)) break;
        uint16_t prog[16] = {0};
        int n = 0;
        for (int i = 0; i < task->num_inputs; i++)
            prog[n++] = PCA_ENC_I(PCA_OP_IN, i + 1, task->input_ports[i]);
        for (uint16_t insn : s.kernel) prog[n++] = insn;
        prog[n++] = PCA_ENC_I(PCA_OP_OUT, s.out_reg, task->output_ports[0]);
        prog[n++] = PCA_ENC_R(PCA_OP_HLT, 0, 0, 0);
        if (task_evaluate(task, prog, n) != task->num_tests) {
            set_err("internal: a GPU solution failed the VM re-check");
            return PCAGB_ELIMIT;
        }
        memcpy(sol_progs + (size_t)stored * 16, prog, sizeof prog);
        if (sol_lens) sol_lens[stored] = n;
        stored++;
    }
    tr.res.stored = stored;
    return PCAGB_OK;
}

/* The recording pass over the levels of a solved task (see pcagb_record). */
int record_levels(pcagb_engine *e, const task_spec_t *task, const TaskRun &tr,
                  const uint16_t *progs, const int *lens, int nprogs, uint32_t task_id,
                  int neg_stride, const char *dir, pcagb_record_stats_t *st)
{
    const GenTables &gt = gen_tables();
    const int K = tr.optimal_depth;
    if ((int)e->levels.size() < K + 1) {
        set_err("internal: levels 0..%d are not built", K);
        return PCAGB_ELIMIT;
    }
    /* states on the optimal programs' paths (tools/enumerate.c:480-520) */
    search_ctx_t ctx;
    search_ctx_init(&ctx, task);
    search_state_t root;
    search_state_init_root(&ctx, &root);
    std::vector<std::unordered_set<uint64_t>> opt(K + 1);
    opt[0].insert(search_state_key_hash64(&ctx, &root));
    for (int si = 0; si < nprogs; si++) {
        search_state_t cur = root;
        const int kl = lens[si] - task->num_inputs - 2;
        for (int k = 0; k < kl; k++) {
            search_state_t next;
            if (!search_state_step(&ctx, &cur, progs[si * 16 + task->num_inputs + k], &next)) break;
            opt[next.depth].insert(search_state_key_hash64(&ctx, &next));
            cur = next;
        }
    }
    st->optimal_states = 0;
    for (auto &o : opt) st->optimal_states += (int)o.size();

    TestPos tp{};
    for (int j = 0; j < tr.T; j++) tp.pos[tr.order[j]] = (uint8_t)j;
    const size_t top0 = e->top;
    auto done = [&](int rc) {
        e->top = top0;
        return rc;
    };
    /* keys of every state, on the device, in the reference's byte order */
    std::vector<std::vector<uint64_t>> keys(K + 1);
    std::vector<uint64_t *> d_key(K + 1), d_oep(K + 1);
    std::vector<std::vector<uint32_t>> parent(K + 1);
    std::vector<std::vector<uint16_t>> cidx(K + 1);
    std::vector<std::vector<uint8_t>> live(K + 1);
    st->visited = 0;
    for (int d = 0; d <= K; d++) {
        const Level &L = e->levels[d];
        st->visited += L.n;
        d_key[d] = (uint64_t *)e->alloc_top(L.n * 8);
        d_oep[d] = (uint64_t *)e->alloc_top(L.n * 8);
        if (!d_key[d] || !d_oep[d]) {
            set_err("arena exhausted recording level %d", d);
            return done(PCAGB_ENOMEM);
        }
        if (e->TPC == 16)
            k_record_keys<16><<<e->grid(4), 256, 0, e->stream>>>(view(L), tp, tr.T, d, d_key[d], d_oep[d]);
        else
            k_record_keys<32><<<e->grid(4), 256, 0, e->stream>>>(view(L), tp, tr.T, d, d_key[d], d_oep[d]);
        int rc = check_launch(e);
        if (rc) return done(rc);
        keys[d].resize(L.n);
        live[d].resize(L.n);
        CK(e_copy(e, keys[d].data(), d_key[d], L.n * 8, cudaMemcpyDeviceToHost, e->stream));
        CK(e_copy(e, live[d].data(), L.live, L.n, cudaMemcpyDeviceToHost, e->stream));
        if (d > 0) {
            parent[d].resize(L.n);
            cidx[d].resize(L.n);
            CK(e_copy(e, parent[d].data(), L.parent, L.n * 4, cudaMemcpyDeviceToHost, e->stream));
            CK(e_copy(e, cidx[d].data(), L.cidx, L.n * 2, cudaMemcpyDeviceToHost, e->stream));
        }
    }
    CK(cudaStreamSynchronize(e->stream));
    /* children of each state are contiguous in the next level (DFS order) */
    std::vector<std::vector<uint64_t>> first(K);
    for (int d = 0; d < K; d++) {
        first[d].assign(e->levels[d].n + 1, 0);
        for (uint32_t p : parent[d + 1]) first[d][p + 1]++;
        for (uint64_t i = 0; i < e->levels[d].n; i++) first[d][i + 1] += first[d][i];
    }
    auto action = [&](int d, uint64_t j) -> uint16_t {
        const uint32_t p = parent[d][j];
        const uint32_t m = (live[d - 1][p] >> 1) & 127u;
        return gt.cand[gt.cand_off[m] + cidx[d][j]];
    };
    /* the depth-first pass (tools/enumerate.c:316-402): states in preorder,
       every non-positive one counted, every neg_stride-th recorded */
    std::vector<std::vector<RecordMeta>> meta(K + 1);
    std::vector<uint64_t> order;  /* preorder of recorded states: depth << 40 | slot */
    std::vector<dataset_edge_record_t> edges;
    uint64_t neg_seen = 0;
    auto visit = [&](auto &&self, int d, uint64_t i, uint16_t act) -> void {
        const uint64_t key = keys[d][i];
        const bool pos = opt[d].count(key) != 0;
        bool rec = pos;
        if (!pos) {
            neg_seen++;
            rec = neg_stride > 0 && neg_seen % (uint64_t)neg_stride == 0;
        }
        if (rec) {
            meta[d].push_back(RecordMeta{(uint32_t)i, act, (uint8_t)(pos ? 1 : 0),
                                         (int8_t)(pos ? K - d : -1)});
            order.push_back((uint64_t)d << 40 | (meta[d].size() - 1));
            if (pos) st->positives++;
            else st->negatives++;
        }
        if (d == K) return;
        for (uint64_t j = first[d][i]; j < first[d][i + 1]; j++) {
            const uint16_t a = action(d + 1, j);
            dataset_edge_record_t er;
            memset(&er, 0, sizeof er);
            er.parent_hash = key;
            er.child_hash = keys[d + 1][j];
            er.action = a;
            er.child_depth = (uint8_t)(d + 1);
            edges.push_back(er);
            self(self, d + 1, j, a);
        }
    };
    visit(visit, 0, 0, (uint16_t)0xFFFF);
    /* the records, serialized on the device */
    std::vector<std::vector<dataset_state_record_t>> recs(K + 1);
    for (int d = 0; d <= K; d++) {
        const uint64_t c = meta[d].size();
        if (!c) continue;
        RecordMeta *dm = (RecordMeta *)e->alloc_top(c * sizeof(RecordMeta));
        dataset_state_record_t *dr =
            (dataset_state_record_t *)e->alloc_top(c * sizeof(dataset_state_record_t));
        if (!dm || !dr) {
            set_err("arena exhausted recording level %d", d);
            return done(PCAGB_ENOMEM);
        }
        CK(e_copy(e, dm, meta[d].data(), c * sizeof(RecordMeta), cudaMemcpyHostToDevice, e->stream));
        CK(cudaMemsetAsync(dr, 0, c * sizeof(dataset_state_record_t), e->stream));
        const Level &L = e->levels[d];
        if (e->TPC == 16)
            k_record_states<16><<<e->grid(4), 256, 0, e->stream>>>(view(L), tp, tr.T, d, task_id, K, dm, c,
                                                                 d_key[d], d_oep[d], dr);
        else
            k_record_states<32><<<e->grid(4), 256, 0, e->stream>>>(view(L), tp, tr.T, d, task_id, K, dm, c,
                                                                 d_key[d], d_oep[d], dr);
        int rc = check_launch(e);
        if (rc) return done(rc);
        recs[d].resize(c);
        CK(e_copy(e, recs[d].data(), dr, c * sizeof(dataset_state_record_t),
                  cudaMemcpyDeviceToHost, e->stream));
    }
    CK(cudaStreamSynchronize(e->stream));
    char path[1024];
    snprintf(path, sizeof path, "%s/states_%06u.bin", dir, task_id);
    FILE *fs = fopen(path, "wb");
    if (!fs) {
        set_err("cannot open %s for writing", path);
        return done(PCAGB_EINVAL);
    }
    for (uint64_t x : order) fwrite(&recs[x >> 40][x & ((1ull << 40) - 1)], sizeof(dataset_state_record_t), 1, fs);
    fclose(fs);
    snprintf(path, sizeof path, "%s/edges_%06u.bin", dir, task_id);
    FILE *fe = fopen(path, "wb");
    if (!fe) {
        set_err("cannot open %s for writing", path);
        return done(PCAGB_EINVAL);
    }
    if (!edges.empty()) fwrite(edges.data(), sizeof(dataset_edge_record_t), edges.size(), fe);
    fclose(fe);
    st->states_written = order.size();
    st->edges_written = edges.size();
    return done(PCAGB_OK);
}

thread_local pcagb_engine *t_default_engine = nullptr;
thread_local uint64_t t_last_explored = 0;

}  // namespace

/* For the branch-mode solver (branch.cu), which runs on the engine's stream
   and device but keeps its own levels. */
cudaStream_t pcagb_internal_stream(pcagb_engine_t *e) { return e->stream; }
int pcagb_internal_device(pcagb_engine_t *e) { return e->device; }

extern "C" {

const char *pcagb_last_error(void) { return g_err.c_str(); }

void pcagb_default_opts(pcagb_opts_t *o)
{
    memset(o, 0, sizeof *o);
    o->max_depth = 4;
    o->min_depth = 0;
    o->split_depth = -1;
    o->oep_mode = PCAGB_OEP_EXACT_LIVE;
}

int pcagb_engine_create(int device, size_t hbm_budget_bytes, pcagb_engine_t **out)
{
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        set_err("no CUDA device: the PCA-16 engine runs only on the GPU");
        return PCAGB_ENODEV;
    }
    if (device < 0 || device >= n) { set_err("bad device %d", device); return PCAGB_EINVAL; }
    pcagb_engine *e = new pcagb_engine();
    int rc = engine_init(e, device, hbm_budget_bytes);
    if (rc) {
        pcagb_engine_destroy(e);
        return rc;
    }
    *out = e;
    return PCAGB_OK;
}

void pcagb_engine_destroy(pcagb_engine_t *e)
{
    if (!e) return;
    cudaSetDevice(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    cudaFree(e->arena);
    cudaFree(e->d_small);
    cudaFree(e->d_status);
    cudaFree(e->d_sol);
    cudaFree(e->d_task_T);
    cudaFree(e->d_task_target);
    cudaFree(e->d_task_active);
    cudaFree(e->d_task_io);
    cudaFree(e->d_hist);
    if (e->h_pin) cudaFreeHost(e->h_pin);
    for (cudaEvent_t ev : {e->ev0, e->ev1, e->ev2, e->ev3, e->evk0, e->evk1})
        if (ev) cudaEventDestroy(ev);
    if (e->stream) cudaStreamDestroy(e->stream);
    delete e;
}

void *pcagb_engine_stream(pcagb_engine_t *e) { return e ? (void *)e->stream : nullptr; }

int pcagb_tuning(pcagb_engine_t *e, pcagb_tuning_t *out)
{
    if (!e || !out) { set_err("null argument"); return PCAGB_EINVAL; }
    memset(out, 0, sizeof *out);
    for (int i = 0; i < 4; i++) out->t_eval_ms[i] = e->t_eval_ms[i];
    out->t_child_ms = e->t_child_ms;
    out->t_child_lean_ms = e->t_child_lean_ms;
    out->t_build_fixed_ms = e->t_build_fixed_ms;
    out->dedup_ratio = e->dedup_ratio;
    memcpy(out->first_tests_ms, e->ft_ms, sizeof e->ft_ms);
    memcpy(out->first_tests_n, e->ft_n, sizeof e->ft_n);
    memcpy(out->chunk_ms, e->ck_ms, sizeof e->ck_ms);
    memcpy(out->chunk_n, e->ck_n, sizeof e->ck_n);
    memcpy(out->chunk_choices, kChunkChoices, sizeof kChunkChoices);
    out->launch_rt_ms = e->launch_rt_ms;
    return PCAGB_OK;
}

int pcagb_device_memory(int device, size_t *free_bytes, size_t *total_bytes)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
        cudaGetLastError();
        set_err("no CUDA device %d", device);
        return PCAGB_ENODEV;
    }
    CK(cudaSetDevice(device));
    CK(cudaMemGetInfo(free_bytes, total_bytes));
    return PCAGB_OK;
}

int pcagb_solve_batch(pcagb_engine_t *e, const task_spec_t *tasks, int ntasks,
                      const pcagb_opts_t *opts, pcagb_result_t *results, uint16_t *sol_progs,
                      int *sol_lens, int sol_cap_per_task)
{
    pcagb_opts_t o;
    if (opts) o = *opts;
    else pcagb_default_opts(&o);
    if (!e || !tasks || !results || ntasks < 1) { set_err("null argument"); return PCAGB_EINVAL; }
    if (ntasks > kMaxBatch) { set_err("at most %d tasks per batch", kMaxBatch); return PCAGB_EINVAL; }
    if (o.oep_mode < PCAGB_OEP_NONE || o.oep_mode > PCAGB_OEP_EXACT_LIVE) {
        set_err("bad oep_mode %d", o.oep_mode);
        return PCAGB_EINVAL;
    }
    std::vector<TaskRun> runs(ntasks);
    for (int i = 0; i < ntasks; i++)
        if (!make_run(&tasks[i], o, &runs[i])) return PCAGB_EINVAL;
    int rc = run_batch(e, runs, o);
    if (rc) return rc;
    for (int i = 0; i < ntasks; i++) {
        uint16_t *p = sol_progs ? sol_progs + (size_t)i * sol_cap_per_task * 16 : nullptr;
        int *l = sol_lens ? sol_lens + (size_t)i * sol_cap_per_task : nullptr;
        rc = emit_solutions(&tasks[i], o, runs[i], p, l, sol_cap_per_task);
        if (rc) return rc;
        results[i] = runs[i].res;
    }
    return PCAGB_OK;
}

int pcagb_solve(pcagb_engine_t *e, const task_spec_t *task, const pcagb_opts_t *opts,
                pcagb_result_t *res, uint16_t *sol_progs, int *sol_lens, int sol_cap)
{
    return pcagb_solve_batch(e, task, 1, opts, res, sol_progs, sol_lens, sol_cap);
}

namespace {
struct DoneCtx {
    const task_spec_t *tasks;
    const pcagb_opts_t *o;
    std::vector<TaskRun> *runs;
    pcagb_result_t *results;
    uint16_t *sol_progs;
    int *sol_lens;
    int cap;
    pcagb_done_cb cb;
    void *user;
    int rc;
};

void deliver(int i, void *p)
{
    DoneCtx &c = *(DoneCtx *)p;
    TaskRun &tr = (*c.runs)[i];
    uint16_t *sp = c.sol_progs ? c.sol_progs + (size_t)i * c.cap * 16 : nullptr;
    int *sl = c.sol_lens ? c.sol_lens + (size_t)i * c.cap : nullptr;
    int rc = emit_solutions(&c.tasks[i], *c.o, tr, sp, sl, c.cap);
    if (rc && !c.rc) c.rc = rc;
    c.results[i] = tr.res;
    if (c.cb) c.cb(i, &c.results[i], c.user);
}
}  // namespace

/* For the solve server (server.cu): an engine without an arena of its own,
   and a batched solve on an arena slice the caller owns (each task with its
   own depth limit), results delivered per task as they are decided. */
int pcagb_internal_engine_create_bare(int device, pcagb_engine_t **out)
{
    if (!out) { set_err("null argument"); return PCAGB_EINVAL; }
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
        cudaGetLastError();
        set_err("no CUDA device %d: the PCA-16 engine runs only on the GPU", device);
        return PCAGB_ENODEV;
    }
    pcagb_engine *e = new pcagb_engine();
    int rc = engine_init(e, device, kArenaExternal);
    if (rc) {
        pcagb_engine_destroy(e);
        return rc;
    }
    *out = e;
    return PCAGB_OK;
}

int pcagb_internal_solve_batch_arena(pcagb_engine_t *e, void *arena, size_t bytes,
                                     const task_spec_t *tasks, const int *max_depths, int ntasks,
                                     const pcagb_opts_t *opts, pcagb_result_t *results,
                                     uint16_t *sol_progs, int *sol_lens, int cap,
                                     pcagb_done_cb on_done, void *user)
{
    if (!e || !arena || !tasks || !max_depths || !results || ntasks < 1 || !opts) {
        set_err("null argument");
        return PCAGB_EINVAL;
    }
    if (ntasks > kMaxBatch) { set_err("at most %d tasks per batch", kMaxBatch); return PCAGB_EINVAL; }
    std::vector<TaskRun> runs(ntasks);
    pcagb_opts_t o = *opts;
    for (int i = 0; i < ntasks; i++) {
        o.max_depth = max_depths[i];
        if (!make_run(&tasks[i], o, &runs[i])) return PCAGB_EINVAL;
    }
    /* the arena's allocations start on 256-byte boundaries (the kernels'
       16-byte pieces and vector loads rely on it): align a supplied base */
    const uintptr_t base = (uintptr_t)arena, aligned = (base + 255) & ~uintptr_t(255);
    if (bytes < aligned - base) { set_err("arena of %zu bytes", bytes); return PCAGB_EINVAL; }
    e->arena = (char *)aligned;
    e->cap = (bytes - (aligned - base)) & ~size_t(255);
    DoneCtx c{tasks, &o, &runs, results, sol_progs, sol_lens, cap, on_done, user, 0};
    int rc = run_batch(e, runs, o, deliver, &c);
    e->arena = nullptr;
    e->cap = e->top = e->bottom = 0;
    return rc ? rc : c.rc;
}

int pcagb_solve_batch_cb(pcagb_engine_t *e, const task_spec_t *tasks, int ntasks,
                         const pcagb_opts_t *opts, pcagb_result_t *results, uint16_t *sol_progs,
                         int *sol_lens, int sol_cap_per_task, pcagb_done_cb on_done, void *user)
{
    pcagb_opts_t o;
    if (opts) o = *opts;
    else pcagb_default_opts(&o);
    if (!e || !tasks || !results || ntasks < 1) { set_err("null argument"); return PCAGB_EINVAL; }
    if (ntasks > kMaxBatch) { set_err("at most %d tasks per batch", kMaxBatch); return PCAGB_EINVAL; }
    std::vector<TaskRun> runs(ntasks);
    for (int i = 0; i < ntasks; i++)
        if (!make_run(&tasks[i], o, &runs[i])) return PCAGB_EINVAL;
    DoneCtx c{tasks, &o, &runs, results, sol_progs, sol_lens, sol_cap_per_task, on_done, user, 0};
    int rc = run_batch(e, runs, o, deliver, &c);
    if (rc) return rc;
    /* the batch totals are known only now */
    for (int i = 0; i < ntasks; i++) results[i] = runs[i].res;
    return c.rc;
}

int pcagb_solve_ordered(pcagb_engine_t *e, const task_spec_t *task, const pcagb_opts_t *opts,
                        pcagb_order_cb order, void *user, uint64_t chunk, pcagb_result_t *res,
                        uint16_t *sol_progs, int *sol_lens, int sol_cap)
{
    pcagb_opts_t o;
    if (opts) o = *opts;
    else pcagb_default_opts(&o);
    if (!e || !task || !res) { set_err("null argument"); return PCAGB_EINVAL; }
    std::vector<TaskRun> runs(1);
    if (!make_run(task, o, &runs[0])) return PCAGB_EINVAL;
    OrderSpec spec{order, user, chunk};
    int rc = run_batch(e, runs, o, nullptr, nullptr, &spec);
    if (rc) return rc;
    rc = emit_solutions(task, o, runs[0], sol_progs, sol_lens, sol_cap);
    *res = runs[0].res;
    return rc;
}

int pcagb_record(pcagb_engine_t *e, const task_spec_t *task, int max_depth, uint32_t task_id,
                 int neg_stride, const char *dir, pcagb_record_stats_t *stats)
{
    if (!e || !task || !dir) { set_err("null argument"); return PCAGB_EINVAL; }
    pcagb_record_stats_t st;
    memset(&st, 0, sizeof st);
    st.optimal_depth = -1;
    pcagb_opts_t o;
    pcagb_default_opts(&o);
    o.max_depth = max_depth;
    o.oep_mode = PCAGB_OEP_EXACT;
    o.count_levels = 1;
    std::vector<TaskRun> runs(1);
    if (!make_run(task, o, &runs[0])) return PCAGB_EINVAL;
    int rc = run_batch(e, runs, o);
    if (rc) return rc;
    const int cap = 100;  /* the reference's MAX_SOLUTIONS */
    std::vector<uint16_t> progs((size_t)cap * 16);
    std::vector<int> lens(cap);
    rc = emit_solutions(task, o, runs[0], progs.data(), lens.data(), cap);
    if (rc) return rc;
    st.optimal_depth = runs[0].optimal_depth;
    if (st.optimal_depth >= 0)
        rc = record_levels(e, task, runs[0], progs.data(), lens.data(), runs[0].res.stored, task_id,
                           neg_stride, dir, &st);
    if (stats) *stats = st;
    if (rc) return rc;
    return st.optimal_depth >= 0 ? 0 : 1;
}

int pcagb_complete(pcagb_engine_t *e, const search_ctx_t *ctx, const search_state_t *start,
                   int max_depth, uint16_t *solution_insns, int *solution_len,
                   uint64_t *states_explored)
{
    if (!e || !ctx || !start || !solution_len) { set_err("null argument"); return PCAGB_EINVAL; }
    *solution_len = 0;
    if (states_explored) *states_explored = 0;
    int max_r = max_depth - (int)start->depth;
    if (max_r > SEARCH_MAX_DEPTH) max_r = SEARCH_MAX_DEPTH;
    std::vector<TaskRun> runs(1);
    TaskRun &tr = runs[0];
    tr.root = *start;
    tr.T = ctx->num_tests;
    if (tr.T < 1 || tr.T > MAX_TESTS) { set_err("bad test count"); return PCAGB_EINVAL; }
    for (int t = 0; t < tr.T; t++) tr.target[t] = ctx->task.tests[t].out[0];
    /* depth 0: the start state already solves */
    for (uint32_t r = 1; r < 8; r++) {
        if (!((start->live >> r) & 1u)) continue;
        bool ok = true;
        for (int t = 0; t < tr.T && ok; t++) ok = start->regs[t][r] == tr.target[t];
        if (ok) return 1;
    }
    if (max_r <= 0) return 0;
    pcagb_opts_t o;
    pcagb_default_opts(&o);
    o.min_depth = 1;
    o.max_depth = max_r;
    o.first_only = 1;
    tr.max_depth = max_r;
    tr.min_depth = 1;
    int rc = run_batch(e, runs, o);
    if (rc) return rc;
    uint64_t explored = 0;
    for (int k = 0; k < PCAGB_MAXD; k++) explored += tr.res.candidates[k];
    if (states_explored) *states_explored = explored;
    if (tr.optimal_depth < 0 || tr.sols.empty()) return 0;
    const RawSol &s = tr.sols.front();
    for (size_t i = 0; i < s.kernel.size(); i++) solution_insns[i] = s.kernel[i];
    *solution_len = (int)s.kernel.size();
    return 1;
}

int search_exhaustive_complete(const search_ctx_t *ctx, const search_state_t *start, int max_depth,
                               uint16_t *solution_insns, int *solution_len)
{
    if (!t_default_engine) {
        int rc = pcagb_engine_create(0, 0, &t_default_engine);
        if (rc) {
            fprintf(stderr, "search_exhaustive_complete: %s\n", pcagb_last_error());
            *solution_len = 0;
            return rc;
        }
    }
    uint64_t explored = 0;
    int rc = pcagb_complete(t_default_engine, ctx, start, max_depth, solution_insns, solution_len,
                            &explored);
    t_last_explored = explored;
    if (rc < 0) fprintf(stderr, "search_exhaustive_complete: %s\n", pcagb_last_error());
    return rc;
}

uint64_t search_exhaustive_states_explored(void) { return t_last_explored; }

}  // extern "C"
