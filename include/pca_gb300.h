/*
 * pca_gb300.h -- C ABI of libpcagb.so, the GB300-native PCA-16
 * superoptimizer engine.
 *
 * Part 1 is a drop-in for the reference's libpca.so (Makefile:23-24), the
 * library the reference's Python binds through ctypes
 * (python/search_eval.py:74-188). Same symbol names, same argument meaning,
 * same return codes, same struct layouts byte for byte. Each declaration
 * cites the reference declaration it replaces.
 *
 * Part 2 is the GPU engine (pcagb_*): the exhaustive iterative-deepening
 * solver whose hot path runs as CUDA kernels on one GB300. The reference
 * has no library interface for its GPU path (gpu/hybrid.cu is a standalone
 * program, gpu/hybrid.cu:631-836); these entry points are what that
 * program's main loop would bind.
 *
 * Plain C types and pointers only. The caller owns every buffer.
 */
#ifndef PCA_GB300_H
#define PCA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------- Part 1: libpca.so ABI ---------------------------------- */

#define PCA_NUM_REGS    8     /* src/pca.h:25 */
#define PCA_MEM_SIZE    256
#define PCA_PROG_SIZE   256
#define PCA_STACK_DEPTH 16
#define PCA_NUM_PORTS   8
#define MAX_TESTS       32    /* tasks/spec.h:17 */
#define MAX_IO_PORTS    8     /* tasks/spec.h:18 */
#define SEARCH_MAX_DEPTH 16   /* src/search_state.h:17 */

#define PCA_RUNNING 0
#define PCA_HALTED  1
#define PCA_TIMEOUT 2
#define PCA_FAULT   3

/* src/pca.h:105-120 */
typedef struct pca_vm {
    uint16_t r[PCA_NUM_REGS];
    uint16_t mem[PCA_MEM_SIZE];
    uint16_t prog[PCA_PROG_SIZE];
    uint8_t  pc;
    uint8_t  sp;
    uint16_t stack[PCA_STACK_DEPTH];
    uint8_t  flags;
    uint8_t  status;
    uint64_t cycles;
    uint16_t ports[PCA_NUM_PORTS];
    void (*on_write)(struct pca_vm *vm, uint8_t port, uint16_t val);
    void (*on_read)(struct pca_vm *vm, uint8_t port);
} pca_vm_t;

/* tasks/spec.h:20-34 */
typedef struct {
    uint16_t in[MAX_IO_PORTS];
    uint16_t out[MAX_IO_PORTS];
} test_case_t;

typedef struct {
    char     name[64];
    uint64_t max_cycles;
    uint8_t  input_ports[MAX_IO_PORTS];
    int      num_inputs;
    uint8_t  output_ports[MAX_IO_PORTS];
    int      num_outputs;
    test_case_t tests[MAX_TESTS];
    int      num_tests;
} task_spec_t;

/* src/search_state.h:20-25 */
typedef struct {
    uint16_t regs[MAX_TESTS][PCA_NUM_REGS];
    uint8_t  flags[MAX_TESTS];
    uint8_t  live;
    uint8_t  depth;
} search_state_t;

/* src/search_state.h:28-35 */
typedef struct {
    task_spec_t task;
    uint8_t num_tests;
    uint8_t num_inputs;
    uint8_t num_outputs;
    uint8_t input_regs[MAX_IO_PORTS];
    uint8_t output_port;
} search_ctx_t;

/* src/search_state.h:38-52 (576-byte label record) */
typedef struct {
    uint64_t state_hash;
    uint64_t oep_hash;
    uint32_t task_id;
    uint16_t parent_action;
    uint8_t  depth;
    uint8_t  budget_left;
    uint8_t  live;
    uint8_t  can_finish_optimally;
    int8_t   remaining_steps;
    uint8_t  _pad[2];
    uint16_t regs[MAX_TESTS][PCA_NUM_REGS];
    uint8_t  flags[MAX_TESTS];
} dataset_state_record_t;

/* src/search_state.h:54-61 (24-byte edge record of the recording pass) */
typedef struct {
    uint64_t parent_hash;
    uint64_t child_hash;
    uint16_t action;
    uint8_t  child_depth;
    uint8_t  _pad[5];
} dataset_edge_record_t;

/* VM: src/pca.h:123-127 */
void pca_init(pca_vm_t *vm);
void pca_load(pca_vm_t *vm, const uint16_t *prog, size_t len);
void pca_step(pca_vm_t *vm);
int  pca_run(pca_vm_t *vm, uint64_t max_cycles);
/* src/pca.h:136-139: "%-4s ..." text of one instruction */
void pca_disasm(uint16_t insn, char *buf, size_t len);
void pca_disasm_prog(const uint16_t *prog, int count);

/* Tasks: tasks/spec.h:37-46. task_load returns 0 / -1 (message on stderr). */
int  task_load(const char *path, task_spec_t *spec);
int  task_evaluate(const task_spec_t *spec, const uint16_t *prog, int prog_len);
void task_print(const task_spec_t *spec);

/* Search state: src/search_state.h:66-131 */
int  search_ctx_init(search_ctx_t *ctx, const task_spec_t *task);         /* 0 / -1 */
void search_state_init_root(const search_ctx_t *ctx, search_state_t *s);
int  search_state_step(const search_ctx_t *ctx, const search_state_t *src,
                       uint16_t insn, search_state_t *dst);               /* 1 ok / 0 illegal */
uint64_t search_state_oep_hash64(const search_ctx_t *ctx, const search_state_t *s);
uint64_t search_state_key_hash64(const search_ctx_t *ctx, const search_state_t *s);
uint8_t  search_state_leaf_outputs(const search_ctx_t *ctx, const search_state_t *s);
void search_state_serialize(const search_ctx_t *ctx, const search_state_t *s,
                            uint32_t task_id, uint16_t parent_action,
                            uint8_t target_depth, uint8_t can_finish_optimally,
                            int8_t remaining_steps, dataset_state_record_t *out);
int  search_gen_candidates_branchless(uint16_t *out, int max, const search_state_t *s);
/* src/search_state.h:108-125. GPU-backed here: returns 1 and the shortest
 * completion (the lexicographically first in candidate order among the
 * shortest) or 0 if none exists within max_depth. Reentrant per thread. */
int  search_exhaustive_complete(const search_ctx_t *ctx, const search_state_t *start,
                                int max_depth, uint16_t *solution_insns,
                                int *solution_len);
/* src/search_state.h:129: states (children) the last completion evaluated */
uint64_t search_exhaustive_states_explored(void);
void search_state_dump(const search_ctx_t *ctx, const search_state_t *s, void *fp);

/* ---------------- Part 2: GPU engine ------------------------------------- */

/* Pruning key of the exact observational-equivalence pruner (OEP). */
#define PCAGB_OEP_NONE       0 /* no pruning: every child kept (small cases) */
#define PCAGB_OEP_EXACT      1 /* key = regs+flags (the reference's key,
                                  tools/enumerate.c:379-384), exact compare,
                                  first child in DFS order represents a key */
#define PCAGB_OEP_EXACT_LIVE 2 /* key = regs+flags+live, exact compare
                                  (default: order independent, sound) */

/* Error codes (negative returns). */
#define PCAGB_OK            0
#define PCAGB_EINVAL       -1  /* bad task or options */
#define PCAGB_ENOMEM       -2  /* HBM budget too small for the split chosen */
#define PCAGB_ECUDA        -3  /* CUDA runtime error (see pcagb_last_error) */
#define PCAGB_ELIMIT       -4  /* a device-side limit was hit (table full,
                                  bounded wait expired); the result is void */
#define PCAGB_ENODEV       -5  /* no CUDA device */

typedef struct pcagb_engine pcagb_engine_t;

typedef struct {
    int max_depth;      /* largest kernel depth K tried (IDDFS 0..max_depth) */
    int min_depth;      /* 0: start with the root check (K = 0, a live
                           register already holding the target); > 0: skip
                           it. Depths 1..max_depth are always searched.      */
    int split_depth;    /* deepest level built with OEP; -1 = automatic      */
    int oep_mode;       /* PCAGB_OEP_*                                       */
    int count_levels;   /* 1: build every level up to K with OEP so that the
                           reference's per-depth counters are reproduced     */
    int first_only;     /* 1: return only the first optimal program in DFS
                           order; the split level is then chosen by the
                           engine's autotuner (the answer does not depend on
                           it). 0: every program found at the optimal depth
                           from the deepest level that fits                  */
    /* Launch choices of the suffix stages; 0 = chosen by the autotuner
       from costs it measures. None changes an answer.                       */
    int first_tests;    /* 1..3: tests a lane checks a value class on before
                           the warp checks its survivors on every test       */
    int suffix_chunk;   /* 1..64: first suffix instructions per work item of
                           the depth-2 and depth-3 suffix kernels, 1024: a
                           lane per innermost middle instruction there; at
                           depth 1 (past the root) 1 = a warp per prefix,
                           >= 32 = a lane per prefix                         */
    int stage_launch;   /* first-only solves of one task: -1 = one launch per
                           stage; n > 0 = a first launch of n prefixes in DFS
                           order, doubling, stopping at the first launch that
                           holds a solution                                  */
    int shared_gpu;     /* 1: the solve shares the GPU with other solves (a
                           server's): its stage times measure the mix, so
                           they update none of the autotuner's costs and no
                           launch choice is explored on it                   */
    int full_levels;    /* 1: every level with its register block; 0: the
                           last depth's split level, which only its
                           last-position stage reads, holds links and the
                           first four tests (probes) only                    */
    int reserved[1];
} pcagb_opts_t;

#define PCAGB_MAXD 17
typedef struct {
    int      optimal_depth;            /* -1: none within max_depth          */
    int      stored;                   /* solutions written to the caller    */
    uint64_t total_solutions;          /* solving programs at optimal depth  */
    uint64_t candidates[PCAGB_MAXD];   /* programs decided per target depth  */
    uint64_t evaluations[PCAGB_MAXD];  /* last-instruction value classes run */
    uint64_t tried[PCAGB_MAXD];        /* the reference's "candidates" count
                                          (valid with count_levels)          */
    uint64_t pruned_cum[PCAGB_MAXD];   /* the reference's cumulative "OEP
                                          pruned" (valid with count_levels)  */
    uint64_t level_children[PCAGB_MAXD];
    uint64_t level_survivors[PCAGB_MAXD];
    double   seconds;                  /* wall time of the solve             */
    double   gpu_ms_expand;            /* device time building levels        */
    double   gpu_ms_suffix;            /* device time in the suffix kernels  */
    double   gpu_ms_insert;            /* device time in the OEP insert kernel */
    uint64_t kernel_launches;          /* kernels this solve launched        */
    uint64_t insert_launches;
    uint64_t suffix_launches;
    uint64_t h2d_bytes;                /* host->device bytes this solve copied */
    uint64_t d2h_bytes;                /* device->host bytes                 */
    uint64_t insert_children;          /* children the insert kernels hashed */
    int      split_used;
    int      reserved0;
    /* ordered solves (pcagb_solve_ordered) at the optimal depth: prefixes of
       the split level, prefixes visited up to and including the first chunk
       that held a solution, and the device time that took */
    uint64_t prefixes_at_optimal;
    uint64_t prefixes_to_first;
    double   ms_to_first;
    uint64_t evaluations_run;          /* value-class evaluations the suffix
                                          kernels executed (a class of an
                                          operand pair counts one); below
                                          `evaluations`, which counts every
                                          class of the candidate space       */
    double   gpu_ms_lanes[PCAGB_MAXD]; /* per target depth: device time of the
                                          lane-per-prefix last-position kernel
                                          alone (without the stage's other
                                          passes) where the stage ran it in
                                          one launch, else 0                 */
} pcagb_result_t;

const char *pcagb_last_error(void);
void pcagb_default_opts(pcagb_opts_t *o);

/* One engine per device and host thread; it owns device buffers sized by
 * hbm_budget_bytes (0 = 60% of the device's free memory). */
int  pcagb_engine_create(int device, size_t hbm_budget_bytes, pcagb_engine_t **out);
void pcagb_engine_destroy(pcagb_engine_t *e);

/* Exhaustive shortest-program solve of one task (the loop of
 * gpu/hybrid.cu:699-824 and tools/enumerate.c:624-662). Solutions are full
 * programs (IN scaffold + kernel + OUT + HLT), 16 words each, in DFS order of
 * the reference's candidate generator; at most sol_cap are stored. */
int  pcagb_solve(pcagb_engine_t *e, const task_spec_t *task, const pcagb_opts_t *opts,
                 pcagb_result_t *res, uint16_t *sol_progs, int *sol_lens, int sol_cap);

/* Batched solve: many tasks share every launch (level expansion, OEP,
 * suffix enumeration); a task leaves the search once its optimal depth is
 * proven or its max_depth is reached. results[i] is task i's result; its
 * `seconds` is the time from the call until task i was decided (its
 * time-to-proven-optimal inside the batch), the gpu_ms_* and byte counters
 * are the batch's. Task i's programs go to
 * sol_progs[i * sol_cap_per_task * 16 ...]. At most 8192 tasks. */
int  pcagb_solve_batch(pcagb_engine_t *e, const task_spec_t *tasks, int ntasks,
                       const pcagb_opts_t *opts, pcagb_result_t *results, uint16_t *sol_progs,
                       int *sol_lens, int sol_cap_per_task);

/* The batched solve with early delivery: on_done(i, &results[i], user) is
 * called on the calling thread as soon as task i is decided (its programs
 * are already in sol_progs), not at the end of the batch. A server returns
 * each request's answer from there. */
typedef void (*pcagb_done_cb)(int task, const pcagb_result_t *result, void *user);
int  pcagb_solve_batch_cb(pcagb_engine_t *e, const task_spec_t *tasks, int ntasks,
                          const pcagb_opts_t *opts, pcagb_result_t *results, uint16_t *sol_progs,
                          int *sol_lens, int sol_cap_per_task, pcagb_done_cb on_done, void *user);

/* A device view of the split level a suffix stage starts from, handed to
 * an ordering callback. Valid only during the callback. regs is
 * u16[n][8][tp] (column-major per state), flags u8[n][tp], live u8[n],
 * task u16[n]; task_io is u16[ntasks][3][32] (input 0, input 1, target per
 * test, in the engine's test order) and task_T int32[ntasks]. */
typedef struct {
    const uint16_t *regs;
    const uint8_t  *flags;
    const uint8_t  *live;
    const uint16_t *task;
    uint64_t n;
    int tp;
    int depth;          /* instructions in each prefix */
    int target_depth;   /* K of the stage */
    int ntasks;
    const uint16_t *task_io;
    const int32_t  *task_T;
    void *stream;       /* cudaStream_t to work on */
    double est_stage_ms; /* the engine's estimate of the whole stage's device time
                            (evaluations x measured ms per evaluation) */
} pcagb_level_view_t;

/* Returns a device array of uint32 holding a permutation of 0..n-1 (the
 * order to visit prefixes in; it must stay valid until the stage ends), or
 * NULL for the plain DFS order. */
typedef const uint32_t *(*pcagb_order_cb)(const pcagb_level_view_t *view, void *user);

/* Solve with the suffix stages visiting prefixes in an order chosen by the
 * callback (e.g. by a value network) in launches of `chunk` prefixes,
 * doubling after each launch that finds nothing, and stopping at the first
 * launch of the optimal depth that holds a solution.
 * Exact: every depth below the optimum is still searched completely, so the
 * optimal depth is proven; only the order of work at the optimal depth
 * changes (its programs are those of the visited chunks).
 * opts->split_depth >= 0 starts every stage from that level and calls the
 * callback for each. split_depth = -1 lets the engine choose: a stage it
 * predicts to finish in under 2 ms runs plain from its cheapest level
 * (no callback; its DFS-first solution is kept), the others start from the
 * level that minimises level builds plus a tenth of the stage. */
int  pcagb_solve_ordered(pcagb_engine_t *e, const task_spec_t *task, const pcagb_opts_t *opts,
                         pcagb_order_cb order, void *user, uint64_t chunk,
                         pcagb_result_t *res, uint16_t *sol_progs, int *sol_lens, int sol_cap);

/* IDDFS completion from an arbitrary branchless state (the GPU form of
 * search_exhaustive_complete, src/search_state.c:418-453). Returns 1 found /
 * 0 none / negative error. */
int  pcagb_complete(pcagb_engine_t *e, const search_ctx_t *ctx, const search_state_t *start,
                    int max_depth, uint16_t *solution_insns, int *solution_len,
                    uint64_t *states_explored);

/* The GPU form of `enumerate --record` (tools/enumerate.c:316-355 records,
 * :480-533 optimal state sets, :676-740 the recording pass). Solves the task
 * with the exact pruner (key regs+flags, DFS-first representative, every
 * level built) and, when a program of kernel depth <= max_depth exists,
 * writes <dir>/states_<task_id>.bin and <dir>/edges_<task_id>.bin as the
 * reference's recording pass does: the states its depth-first pass visits
 * at the optimal depth K* (levels 0..K*, in depth-first preorder), every
 * state on the path of one of the first 100 optimal programs (positive,
 * with its remaining steps) and every neg_stride-th other state (negative),
 * as dataset_state_record_t; and one dataset_edge_record_t per visited
 * child. The levels come from HBM; keys, hashes and records are computed on
 * the device. Returns 0 when recorded, 1 when no program exists (nothing
 * written), negative on error. */
typedef struct {
    int      optimal_depth;
    int      optimal_states;    /* distinct path states over all depths */
    uint64_t states_written;
    uint64_t positives;
    uint64_t negatives;
    uint64_t edges_written;
    uint64_t visited;           /* states of levels 0..K* */
} pcagb_record_stats_t;

int  pcagb_record(pcagb_engine_t *e, const task_spec_t *task, int max_depth, uint32_t task_id,
                  int neg_stride, const char *dir, pcagb_record_stats_t *stats);

/* The reference solver's branch mode (its default, without --no-branch;
 * tools/enumerate.c:204-455): kernels may use CMP, forward BR (cond 1..6,
 * offsets up to the end of the kernel), DIV and MOD besides the branchless
 * set, with the reference's candidate rules and its pruner (key: registers
 * and flags of every test after the partial program; BR children never
 * pruned; first child in depth-first order kept), exact here. Every level
 * of each depth is built on the engine's stream, so the per-depth counters
 * (tried, pruned_cum) are the reference's, up to the 100th solution at the
 * optimal depth as its walk stops there; the first sol_cap programs in
 * depth-first order are returned. Errors: see pcagb_branch_last_error. */
int  pcagb_solve_branch(pcagb_engine_t *e, const task_spec_t *task, int max_depth,
                        pcagb_result_t *res, uint16_t *sol_progs, int *sol_lens, int sol_cap);
/* The same with the size rule of the last position explicit: when a depth's
 * last position has more than last_level_max_children children (default
 * 2^26), its level is not built; the solving children are found directly
 * and kept when they are the depth-first first of their key (the same
 * programs), and that depth's counters are the engine's (split_used = K-1). */
int  pcagb_solve_branch_ex(pcagb_engine_t *e, const task_spec_t *task, int max_depth,
                           uint64_t last_level_max_children, pcagb_result_t *res,
                           uint16_t *sol_progs, int *sol_lens, int sol_cap);
/* Branch mode with the reference hybrid solver's stopping rule
 * (gpu/hybrid.cu:524-555: the search ends at the first batch of prefixes
 * with a solution): every depth below the optimum is searched completely;
 * at each depth the last position is searched without building its level,
 * over the parents in depth-first order in launches of 1/64 of them,
 * doubling, and the depth ends at the first launch that holds a solution.
 * The optimal depth is the same as pcagb_solve_branch's, and so are the
 * programs returned: the first in depth-first order, up to sol_cap, all
 * from that launch. tried[K] / candidates[K] count the children built
 * plus the last-position children of the parents visited. */
int  pcagb_solve_branch_first(pcagb_engine_t *e, const task_spec_t *task, int max_depth,
                              pcagb_result_t *res, uint16_t *sol_progs, int *sol_lens,
                              int sol_cap);
const char *pcagb_branch_last_error(void);

/* The CUDA stream (cudaStream_t) every kernel of this engine runs on, so a
 * caller can time a solve with events on that stream. */
void *pcagb_engine_stream(pcagb_engine_t *e);

/* The autotuner's measured costs on this engine's device: device ms per
 * value-class evaluation of each suffix depth (t_eval_ms) and per child of a
 * level build, and for each suffix depth s the cost of each launch choice
 * (first_tests 1..3 at [s][1..3], work-item shape c at [s][c]: for s >= 2
 * chunk_choices[s][c] first instructions per work item, 1024 meaning a lane
 * per innermost middle, for s = 1 the prefixes a warp scans at once, 1 or
 * 32) with the number of stages it was measured on; the host round trip of
 * a chunked launch. */
typedef struct {
    double   t_eval_ms[4];
    double   t_child_ms;
    double   t_build_fixed_ms;
    double   dedup_ratio;
    double   first_tests_ms[4][4];
    int      first_tests_n[4][4];
    double   chunk_ms[4][4];
    int      chunk_n[4][4];
    uint32_t chunk_choices[4][4];
    double   launch_rt_ms;
    double   t_child_lean_ms;          /* per child of a lean level build (the
                                          last stage's split level: probes and
                                          links only)                        */
} pcagb_tuning_t;
int  pcagb_tuning(pcagb_engine_t *e, pcagb_tuning_t *out);

/* Free and total device memory, for sizing engines (a server admits work by
 * free HBM). */
int  pcagb_device_memory(int device, size_t *free_bytes, size_t *total_bytes);

/* Number of generator candidates for a live mask (src/search_state.c:280-330). */
int  pcagb_num_candidates(uint8_t live);

/* ---- Solve without allocating (no counterpart in the reference) ----------
 * For callers that cannot call cudaMalloc -- a process whose device memory
 * belongs to another allocator's pool, latency-critical code that must not
 * risk the synchronisation an allocation can cause, hosts that forbid a
 * plugin from owning device memory. Needs no engine. Enumerates every kernel
 * program of length 1..max_depth straight from the task root and returns the
 * full canonical program set at the optimal length (the programs
 * pcagb_solve returns with split_depth 0, here in no particular order).
 * Scratch is one file-scope static __device__ array of
 * PCAGB_NOALLOC_SCRATCH_BYTES that every GPU loading the library holds until
 * exit; the first call on a device sets it up (call it once before any
 * stream capture). Calls share the array: calls that overlap on the GPU
 * race. max_depth above PCAGB_NOALLOC_MAX_DEPTH, or more solving records
 * than the scratch holds, is rejected (PCAGB_EINVAL / PCAGB_ELIMIT; message
 * in pcagb_noalloc_last_error). Runs on the current device and the given
 * stream (NULL = legacy default stream). Returns 1 found / 0 none /
 * negative error. */
#define PCAGB_NOALLOC_SCRATCH_BYTES (16u << 20)
#define PCAGB_NOALLOC_MAX_DEPTH 3
int  pcagb_solve_small_noalloc(const task_spec_t *task, int max_depth, void *stream,
                               int *optimal_depth, uint64_t *total_solutions,
                               uint16_t *sol_progs, int *sol_lens, int sol_cap);
const char *pcagb_noalloc_last_error(void);

/* ---------------- Part 3: serving ---------------------------------------- */

/* A solve server on one GPU (server.cu). The reference solves one task per
 * process run (tools/enumerate.c, gpu/hybrid.cu:631-836) and has no serving
 * loop; these entry points are what a request loop around that solver would
 * bind. Requests of any input count, test count and depth are submitted as
 * they arrive; a request is admitted as soon as a worker is idle and the
 * device pool holds an arena slice for it (admission by free HBM, in
 * arrival order), solves run concurrently on their own CUDA streams, queued
 * requests found together share one batched solve, and each answer is
 * stored the moment its task is decided. Every wait is on the host, with a
 * timeout. */
typedef struct pcagb_server pcagb_server_t;

typedef struct {
    int      device;
    size_t   pool_bytes;   /* device pool for all solves; 0 = 80% of free memory */
    size_t   arena_bytes;  /* the slice one solve reserves (a batch: up to four) */
    int      workers;      /* solves that may run at once, each on its stream */
    int      max_batch;    /* queued requests one solve may take together */
    int      sol_cap;      /* programs kept per request */
    pcagb_opts_t opts;     /* solve options (default: first_only) */
} pcagb_server_config_t;

typedef struct {
    uint64_t queued;
    uint64_t running_solves;
    uint64_t max_running_solves;
    uint64_t admitted;
    uint64_t finished;
    uint64_t batches;            /* solves run (a solve takes one or more requests) */
    uint64_t pool_bytes;
    uint64_t pool_used;
    uint64_t pool_peak;
    uint64_t pool_largest_free;
} pcagb_server_stats_t;

void pcagb_server_default_config(pcagb_server_config_t *cfg);
int  pcagb_server_create(const pcagb_server_config_t *cfg, pcagb_server_t **out);
/* Queue a solve of the task up to kernel depth max_depth; *id names it. */
int  pcagb_server_submit(pcagb_server_t *s, const task_spec_t *task, int max_depth,
                         uint64_t *id);
/* The next finished request, in the order requests finish: 1 and *id, or 0
 * when none finishes within timeout_s seconds. */
int  pcagb_server_next(pcagb_server_t *s, double timeout_s, uint64_t *id);
/* A finished request's result and first `cap` programs (then forgotten);
 * times[0..3] = submitted, admitted, finished (seconds since the server
 * started) and the number of requests its solve took. Returns 0, or the
 * solve's error code (PCAGB_ENOMEM when the pool cannot hold one arena). */
int  pcagb_server_collect(pcagb_server_t *s, uint64_t id, pcagb_result_t *res,
                          uint16_t *sol_progs, int *sol_lens, int cap, double *times);
int  pcagb_server_stats(pcagb_server_t *s, pcagb_server_stats_t *stats);
/* Takes no new requests, solves the queued ones, then frees everything. */
void pcagb_server_destroy(pcagb_server_t *s);
const char *pcagb_server_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
