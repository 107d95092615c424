/*
 * pca_oracle.h -- CPU restatement of the reference PCA-16 branchless search
 * path. TEST INFRASTRUCTURE ONLY: used by tests/, the smoke check and the CPU
 * baseline leg of bench.py as the checker. Nothing in the product links it.
 *
 * Every function names the reference file:line it restates. Struct layouts
 * restate tasks/spec.h:17-34 and src/search_state.h:20-35 byte for byte so
 * the same ctypes mirrors work for both this oracle and the product library.
 */
#ifndef PCA_ORACLE_H
#define PCA_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAX_TESTS    32   /* tasks/spec.h:17 */
#define ORC_MAX_IO_PORTS 8    /* tasks/spec.h:18 */
#define ORC_NUM_REGS     8    /* src/pca.h:25 */
#define ORC_MAX_DEPTH    16   /* src/search_state.h:17 */

typedef struct {
    uint16_t in[ORC_MAX_IO_PORTS];
    uint16_t out[ORC_MAX_IO_PORTS];
} orc_test_case_t;

typedef struct {                       /* tasks/spec.h:25-34 */
    char     name[64];
    uint64_t max_cycles;
    uint8_t  input_ports[ORC_MAX_IO_PORTS];
    int      num_inputs;
    uint8_t  output_ports[ORC_MAX_IO_PORTS];
    int      num_outputs;
    orc_test_case_t tests[ORC_MAX_TESTS];
    int      num_tests;
} orc_task_t;

typedef struct {                       /* src/search_state.h:20-25 */
    uint16_t regs[ORC_MAX_TESTS][ORC_NUM_REGS];
    uint8_t  flags[ORC_MAX_TESTS];
    uint8_t  live;
    uint8_t  depth;
} orc_state_t;

typedef struct {                       /* src/search_state.h:28-35 */
    orc_task_t task;
    uint8_t num_tests;
    uint8_t num_inputs;
    uint8_t num_outputs;
    uint8_t input_regs[ORC_MAX_IO_PORTS];
    uint8_t output_port;
} orc_ctx_t;

/* OEP modes of orc_enumerate. */
enum {
    ORC_OEP_NONE  = 0,  /* no pruning: the full canonical program set        */
    ORC_OEP_REF32 = 1,  /* the reference's pruner: low 32 bits of FNV-1a-64,
                           2^20-slot table per depth, 32 linear probes,
                           full window = keep (tools/enumerate.c:43-89)       */
    ORC_OEP_EXACT = 2,  /* exact key regs+flags, DFS first-wins              */
    ORC_OEP_EXACT_LIVE = 3, /* exact key regs+flags+live (order independent) */
    ORC_OEP_REF32_AUDIT = 4 /* REF32, plus an exact shadow set that counts the
                               reference's false prunes (32-bit collisions) and
                               missed prunes (probe window full)             */
};

typedef struct {
    int      optimal_depth;               /* -1: none within max_depth        */
    uint64_t tried[ORC_MAX_DEPTH + 1];    /* reference "candidates" per depth  */
    uint64_t pruned_cum[ORC_MAX_DEPTH + 1];/* reference "OEP pruned" (cumul.)  */
    int      sols_at[ORC_MAX_DEPTH + 1];  /* solutions found at each depth     */
    /* OEP survivors per level at the final target depth (level 0 = root).   */
    uint64_t survivors[ORC_MAX_DEPTH + 1];
    uint64_t children[ORC_MAX_DEPTH + 1]; /* children generated per level     */
    int      num_solutions;               /* stored solutions                  */
    uint64_t total_solutions;             /* found, including beyond the cap   */
    uint64_t false_prunes;                /* REF32_AUDIT: pruned, state was new */
    uint64_t missed_prunes;               /* REF32_AUDIT: kept, state was seen  */
} orc_result_t;

/* tasks/spec.c:80-184 */
int  orc_task_load(const char *path, orc_task_t *spec);
/* tasks/spec.c:188-215 with src/vm.c:58-217 */
int  orc_task_evaluate(const orc_task_t *spec, const uint16_t *prog, int len);
/* src/search_state.c:15-45 */
int  orc_ctx_init(orc_ctx_t *ctx, const orc_task_t *task);
void orc_init_root(const orc_ctx_t *ctx, orc_state_t *s);
/* src/search_state.c:49-187 */
int  orc_step(const orc_ctx_t *ctx, const orc_state_t *src, uint16_t insn,
              orc_state_t *dst);
/* src/search_state.c:191-219 */
uint64_t orc_oep_hash64(const orc_ctx_t *ctx, const orc_state_t *s);
uint64_t orc_key_hash64(const orc_ctx_t *ctx, const orc_state_t *s);
/* src/search_state.c:223-239 */
uint8_t orc_leaf_outputs(const orc_ctx_t *ctx, const orc_state_t *s);
/* src/search_state.c:280-330 */
int  orc_gen_candidates(uint16_t *out, int max, uint8_t live);
/* src/search_state.c:339-453 */
int  orc_exhaustive_complete(const orc_ctx_t *ctx, const orc_state_t *start,
                             int max_depth, uint16_t *sol, int *sol_len,
                             uint64_t *states_explored);

/* Iterative deepening of tools/enumerate.c:316-402 and :624-662 (branchless
 * mode) with a selectable pruner. Solutions are full programs
 * (IN scaffold + kernel + OUT + HLT), each padded to 16 words, in DFS order;
 * at most sol_cap are stored (sol_cap < 0 = the reference's cap of 100 and
 * its early stop; sol_cap >= 0 = full traversal of the optimal depth). */
int  orc_enumerate(const orc_task_t *task, int max_depth, int oep_mode,
                   int sol_cap, uint16_t *sol_progs, int *sol_lens,
                   orc_result_t *res);

/* Iterative deepening of the reference's branch mode, its default without
 * --no-branch (tools/enumerate.c:204-260 candidates with CMP, forward BR,
 * DIV and MOD; :262-286 output check; :405-455 search; :624-662 driver):
 * every candidate re-runs the partial program on the VM for every test (100
 * cycles) and is pruned when its registers and flags were seen at that
 * position, BR candidates excepted. oep_mode: ORC_OEP_REF32 (the
 * reference's 32-bit FNV-1a key in its 2^20-slot tables), ORC_OEP_EXACT
 * (the same key compared exactly) or ORC_OEP_NONE. The walk stops at the
 * 100th solution of a depth, as the reference's does. */
int  orc_enumerate_branch(const orc_task_t *task, int max_depth, int oep_mode,
                          uint16_t *sol_progs, int *sol_lens, orc_result_t *res);

/* CPU throughput baseline: the reference algorithm (REF32 pruner) at one
 * fixed kernel depth on nthreads POSIX threads. Work items are the
 * (root candidate, level-1 candidate) pairs, handed out in DFS order from a
 * shared counter; each thread keeps its own OEP tables. No item starts after
 * budget_s seconds. Returns the candidates ("tried") counted; *seconds gets
 * the wall time. */
uint64_t orc_enumerate_sample(const orc_task_t *task, int depth, int nthreads,
                              double budget_s, double *seconds,
                              uint64_t *solutions);

/* Level-synchronous, multi-threaded form of the branchless IDDFS
 * (oracle_levels.c): for each K = 0..max_depth, the kept states of
 * positions 1..S (S = min(K-1, split)) under oep_mode (NONE, EXACT or
 * EXACT_LIVE; the first child in the reference's depth-first order keeps a
 * key) and positions S+1..K without pruning; stops at the first K with a
 * solution. Every solving (kernel, output register) at that K is counted in
 * total_solutions and the first sol_cap are stored in depth-first order.
 * tried[K] counts every generated child of positions 1..K; survivors and
 * children hold levels 0..S. Returns 0, or -1 on bad arguments or when host
 * memory runs out. */
int  orc_enumerate_split(const orc_task_t *task, int max_depth, int split, int oep_mode,
                         int nthreads, int sol_cap, uint16_t *sol_progs, int *sol_lens,
                         orc_result_t *res);

#ifdef __cplusplus
}
#endif
#endif
