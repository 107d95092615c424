/*
 * engine_kernels.cuh -- CUDA kernels of the PCA-16 exhaustive engine.
 *
 * Search levels. Level d holds the distinct states reached by d kernel
 * instructions (level 0 = the task root). A state is stored column-major:
 * regs[n][8][TP] (u16, r0's column kept as zeros), flags[n][TP], live[n],
 * plus the back pointer (parent rank, candidate index) that rebuilds its
 * program. TP is 16 or 32 (test count rounded up), and test slots >= T are
 * zero in every state.
 *
 * Level expansion (the OEP kernel): one warp per parent, one lane per child
 * candidate. Each lane computes the child's new column and flags across all
 * tests, a 64-bit hash of the whole child state (incrementally from the
 * parent's per-column hashes), and inserts a 64-bit slot
 *   [tag: hash bits 40..63][ref + 1: 40 bits]
 * into an open-addressed HBM table, ref = parent_rank << 12 | candidate.
 * On a tag match the two child states are rebuilt and compared in full
 * (every register of every test, flags, and live when it is part of the
 * key), so a hash collision can never merge two different states. Among
 * equal states the smallest ref wins (atomicCAS loop), which is the first
 * child in the reference's DFS order -- the representative the reference's
 * DFS pruner keeps (tools/enumerate.c:379-384). Children that can never be
 * that representative are not inserted at all: same-state siblings of an
 * earlier candidate (bit 31 of the device micro-op), children overwriting a
 * dead-able unread write (deadable_writes) and LDI swaps (ldi_swap); each
 * has an equal state with a smaller ref, so the winners do not change.
 *
 * The winners are then marked in a bitmap indexed by the child's linear
 * index (child_off[parent] + candidate), ranked by a scan, and written out
 * in that order, so every level stays in DFS order.
 *
 * Suffix kernels: one warp per prefix state. The last instruction's value
 * does not depend on its destination (except ADDI), so only value classes
 * are evaluated, and only those that read the last write (the read rule in
 * scan_last): one lane per operand pair, every op of the pair evaluated on
 * the first two tests at once, each survivor checked on all tests by the
 * warp (lane t taking test t, __all_sync deciding). Suffix depths 2 and 3
 * enumerate the middle instructions in the warp, keeping the new columns in
 * spare shared-memory columns 8 and 9.
 */
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "pca_isa.h"
#include "scan.cuh"

namespace pcagb {

constexpr int kWarpsPerBlock = 8;
constexpr int kThreads = kWarpsPerBlock * 32;
constexpr uint64_t kRefMask = (1ull << 40) - 1;
constexpr uint32_t kMaxProbes = 1u << 16;

/* status flags set by kernels (bounded loops that ran out) */
constexpr uint32_t kStatusTableFull = 1u;
constexpr uint32_t kStatusRefOverflow = 2u;

/* Candidate tables, uploaded once per device. */
__constant__ uint32_t c_cand_off[129];
__constant__ uint32_t c_vc_off[129];
__constant__ const uint32_t *c_cand_uop;   /* bit 31: a same-state duplicate of an earlier candidate */
__constant__ const uint32_t *c_vc_uop;
__constant__ const uint16_t *c_vc_first;   /* first candidate index per class */
__constant__ uint32_t c_chunk_off[129];    /* op-uniform runs of candidates */
__constant__ const uint32_t *c_chunks;
__constant__ uint32_t c_vcr_off[128 * 8 + 1]; /* [mask*8 + r]: classes reading r */
__constant__ const uint32_t *c_vcr_uop;    /* their micro-ops */
__constant__ const uint16_t *c_vcr;        /* their indices in the mask's class list */
__constant__ uint32_t c_pr_off[128 * 8 + 1];  /* [mask*8 + r]: the same, by operand pair */
__constant__ const uint32_t *c_pr;         /* a | b << 3 | opmask << 6 | imm << 16 */
__constant__ const uint16_t *c_pr_cls;     /* [entry][10] class index per opmask bit */
__constant__ uint32_t c_pr_ev[128 * 8];    /* [mask*8 + r]: class evaluations of its pair list */
__constant__ const uint32_t *c_ev_sd1;     /* the same in global memory, [mask*8 + 0] = all classes */
__constant__ const uint32_t *c_pr_off_g;   /* c_pr_off in global memory (lanes of different masks) */

/* Per-task parameters of a batch: device arrays indexed by task id. A
   state's task id travels with it through the levels; states of different
   tasks never compare equal. */
struct TaskDev {
    const int32_t *T;          /* tests of each task */
    const uint32_t *target;    /* [task][32] expected outputs */
    const uint8_t *active;     /* task still searched at the current depth */
    int key_live;              /* OEP key includes live */
    int dedup_mid;             /* OEP on: a suffix's middle instruction that
                                  repeats an earlier sibling's state is skipped */
};

struct LevelDev {
    const uint16_t *regs;   /* [n][8][TP] */
    const uint8_t *flags;   /* [n][TP] */
    const uint8_t *live;    /* [n] */
    const uint16_t *task;   /* [n] */
    const uint64_t *child_off; /* [n+1] */
    uint64_t n;
    const uint8_t *rdl;     /* [n] register the state's last instruction wrote (0: root) */
    const uint32_t *parent; /* [n] rank of the parent in the level above */
    const uint8_t *own;     /* [n] registers whose last write is unread and dead-able (below);
                               bit 0: the last instruction is an LDI */
    const uint8_t *twin;    /* [n] 1: an earlier state of the level has the same registers,
                               live mask and task (k_twins) */
    const uint16_t *probe;  /* [n][8][4] r0..r7 on the first four tests, 64 bytes a state */
};

/* A lean level (k_materialize_probe: links and probes, no register block)
   reaches its states' registers through their parents: the level above's
   registers and liveness, and the lean level's own candidate indices.
   up_regs == nullptr: the level is a full one. */
struct LeanDev {
    const uint16_t *up_regs;   /* [n_up][8][TP] */
    const uint8_t *up_live;    /* [n_up] */
    const uint16_t *cidx;      /* [n] candidate index of each state in its parent's list */
};

struct LevelOut {
    uint16_t *regs;
    uint8_t *flags;
    uint8_t *live;
    uint16_t *task;
    uint32_t *parent;
    uint16_t *cidx;
    uint8_t *rdl;
    uint8_t *own;
    uint16_t *probe;
};

/* ---- hashing (a multiply-rotate chain; the table compares full states, so
        the hash only has to spread well) -------------------------------- */

__device__ __forceinline__ uint64_t fmix64(uint64_t x)
{
    x ^= x >> 33;
    x *= 0xFF51AFD7ED558CCDull;
    x ^= x >> 33;
    x *= 0xC4CEB9FE1A85EC53ull;
    x ^= x >> 33;
    return x;
}

__device__ __forceinline__ uint64_t chain(uint64_t h, uint64_t w)
{
    h = (h ^ w) * 0x9E3779B97F4A7C15ull;
    return (h << 27) | (h >> 37);
}

__device__ __forceinline__ uint64_t col_final(uint32_t r, uint64_t h)
{
    return fmix64(h + (uint64_t)r * 0xD6E8FEB86659FD93ull);
}

__device__ __forceinline__ uint64_t live_final(uint32_t live)
{
    return fmix64(0x5851F42D4C957F2Dull ^ live);
}

__device__ __forceinline__ uint64_t task_final(uint32_t task)
{
    return fmix64(0x9E3779B97F4A7C15ull * (task + 1));
}

template <int TPC, typename E>
__device__ __forceinline__ uint64_t hash_column(const E *col)
{
    uint64_t h = 0x243F6A8885A308D3ull;
#pragma unroll
    for (int t = 0; t < TPC; t += 4) {
        uint64_t w = (uint64_t)col[t] | ((uint64_t)col[t + 1] << 16) |
                     ((uint64_t)col[t + 2] << 32) | ((uint64_t)col[t + 3] << 48);
        h = chain(h, w);
    }
    return h;
}

/* Reads: does micro-op u read register r (1..7)? */
__device__ __forceinline__ bool uop_reads(uint32_t u, uint32_t r)
{
    return UOP_A(u) == r || UOP_B(u) == r;
}

/* Dead writes. In a state's path, a write to register w that no later
   instruction has read yet, made by an instruction z that is not the first
   kept sibling writing w (the lowest-ranked kept child of z's parent that
   writes w), is dead-able: a child y that is not an LDI and overwrites w
   without reading it reaches a state (registers, y's flags, live) that the
   same path with the first sibling in z's place reaches too, by a smaller
   ref (every instruction after z is the same candidate under the same
   liveness mask, and none reads w). Such a child is never the DFS-first
   representative, so the insert kernel skips it and the table's winners,
   and every level, are unchanged. A state keeps these registers in `own`
   (writes older than its last instruction); its last write is dead-able
   when the state is not the first kept sibling writing it (fcr_up, the
   first-child ranks of the level above). */
__device__ __forceinline__ uint32_t deadable_writes(const LevelDev &P, const uint32_t *fcr_up,
                                                    uint64_t q)
{
    if (!fcr_up) return 0;
    uint32_t W = P.own[q] & 0xFEu;
    const uint32_t w = P.rdl[q];
    if (w && fcr_up[(uint64_t)P.parent[q] * 8 + w] != (uint32_t)q) W |= 1u << w;
    return W;
}

/* LDI swaps. When a state's last instruction is an LDI (bit 0 of `own`)
   writing register y, a child x that neither reads nor writes y reaches the
   state of the path with x and the LDI in the other order (the LDI keeps
   the flags, so both end with x's). That path is the smaller ref when x
   comes first in the generator's order: every ALU op precedes every LDI,
   and an LDI precedes another when its register is lower. Such a child is
   never the DFS-first representative; the insert kernel skips it. */
__device__ __forceinline__ bool ldi_swap(uint32_t u, uint32_t last_ldi_reg)
{
    if (!last_ldi_reg) return false;
    const uint32_t op = UOP_OP(u), rd = UOP_RD(u);
    if (rd == last_ldi_reg || uop_reads(u, last_ldi_reg)) return false;
    if (op == PCA_OP_LDI) return rd < last_ldi_reg;
    return op != PCA_OP_ADDI;
}

/* ---- shared-memory view of one state per warp ---------------------------- */

template <int TPC>
struct WarpState {
    uint32_t R[10][TPC + 1];  /* columns r0..r7 + 2 spare; +1 word pad */
    uint32_t F[TPC];
    uint64_t colh[8];         /* colh[r] = col_final(r, hash(col r)), r >= 1 */
};

/* ---- level expansion: insert every child into the exact table ------------ */

/* One warp's shared memory in the insert kernel: its parent (16-bit columns,
   a row stride of TPC + 2 halves so that lanes reading different operand
   columns of one test hit different banks) and the new column and flags of
   each lane's child in the current chunk, which the warp-wide compares read
   instead of recomputing them. */
template <int TPC>
struct InsertState {
    uint64_t colh[8];           /* colh[r] = col_final(r, hash(col r)), r >= 1 */
    uint64_t flagsA[TPC / 16][32]; /* [word][lane]: the lane's child flags, 4 bits a test */
    uint16_t R[8][TPC + 2];
    uint16_t colA[TPC][33];     /* [test][lane]: odd stride, a test row per lane is conflict free */
    uint8_t F[TPC];
};

template <int TPC>
__device__ __forceinline__ void load_insert_state(InsertState<TPC> &ws, const uint16_t *regs,
                                                  const uint8_t *flags, uint64_t q, int lane)
{
    if (lane < TPC) {
        const uint16_t *src = regs + q * 8 * TPC + lane;
#pragma unroll
        for (int r = 0; r < 8; r++) ws.R[r][lane] = src[r * TPC];
        ws.F[lane] = flags[q * TPC + lane];
    }
}

/* The op is a template parameter here: a warp expands a run of candidates
   that share one op, so the switch is resolved at compile time and the
   lanes never diverge on it. */
template <int OP>
__device__ __forceinline__ uint32_t alu_t(uint32_t a, uint32_t b, uint32_t imm)
{
    if constexpr (OP == PCA_OP_ADD) return (a + b) & 0xFFFFu;
    else if constexpr (OP == PCA_OP_SUB) return (a - b) & 0xFFFFu;
    else if constexpr (OP == PCA_OP_MUL) return (a * b) & 0xFFFFu;
    else if constexpr (OP == PCA_OP_AND) return a & b;
    else if constexpr (OP == PCA_OP_OR) return a | b;
    else if constexpr (OP == PCA_OP_XOR) return a ^ b;
    else if constexpr (OP == PCA_OP_SHL) return (a << (b & 15u)) & 0xFFFFu;
    else if constexpr (OP == PCA_OP_SHR) return a >> (b & 15u);
    else if constexpr (OP == PCA_OP_ASR) return (uint32_t)(uint16_t)((int16_t)(uint16_t)a >> (b & 15u));
    else if constexpr (OP == PCA_OP_LDI) return imm;
    else return (a + (uint32_t)(int32_t)(int8_t)(uint8_t)imm) & 0xFFFFu; /* ADDI */
}

template <int OP>
__device__ __forceinline__ uint32_t flags_t(uint32_t a, uint32_t b, uint32_t imm, uint32_t res,
                                            uint32_t old)
{
    if constexpr (OP == PCA_OP_LDI) return old;
    else if constexpr (OP == PCA_OP_ADD || OP == PCA_OP_SUB || OP == PCA_OP_MUL ||
                       OP == PCA_OP_ADDI)
        return pca_alu_flags(OP, a, b, imm, res, old);
    else return pca_zn(res);
}

/* Hash of the child's new column (chain over 4 tests per word) and of its
   flags (16 tests per word), tests >= T contributing zeros; the column and
   the flags are also left in the warp's shared memory for the compares. The
   loop over word groups is kept rolled: eleven op variants of a fully
   unrolled loop overflow the instruction cache. */
template <int TPC, int OP>
__device__ __forceinline__ void child_hashes(InsertState<TPC> &ws, uint32_t ra, uint32_t rb,
                                             uint32_t imm, int T, int lane, uint64_t &h,
                                             uint64_t &hf)
{
    h = 0x243F6A8885A308D3ull;
    hf = 0x13198A2E03707344ull;
    uint64_t wf = 0;
#pragma unroll 1
    for (int t0 = 0; t0 < TPC; t0 += 4) {
        uint64_t w = 0;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int t = t0 + j;
            const uint32_t a = ws.R[ra][t], b = ws.R[rb][t];
            uint32_t res = alu_t<OP>(a, b, imm);
            uint32_t f = flags_t<OP>(a, b, imm, res, ws.F[t]);
            if (t >= T) { res = 0; f = 0; }
            ws.colA[t][lane] = (uint16_t)res;
            w |= (uint64_t)res << (16 * j);
            wf |= (uint64_t)f << (4 * (t & 15));
        }
        h = chain(h, w);
        if ((t0 & 15) == 12) {
            hf = chain(hf, wf);
            ws.flagsA[t0 >> 4][lane] = wf;
            wf = 0;
        }
    }
}

template <int TPC>
__device__ __forceinline__ void child_hashes_any(uint32_t op, InsertState<TPC> &ws, uint32_t ra,
                                                 uint32_t rb, uint32_t imm, int T, int lane,
                                                 uint64_t &h, uint64_t &hf)
{
    switch (op) {
    case PCA_OP_ADD: child_hashes<TPC, PCA_OP_ADD>(ws, ra, rb, imm, T, lane, h, hf); break;
    case PCA_OP_SUB: child_hashes<TPC, PCA_OP_SUB>(ws, ra, rb, imm, T, lane, h, hf); break;
    case PCA_OP_MUL: child_hashes<TPC, PCA_OP_MUL>(ws, ra, rb, imm, T, lane, h, hf); break;
    case PCA_OP_AND: child_hashes<TPC, PCA_OP_AND>(ws, ra, rb, imm, T, lane, h, hf); break;
    case PCA_OP_OR: child_hashes<TPC, PCA_OP_OR>(ws, ra, rb, imm, T, lane, h, hf); break;
    case PCA_OP_XOR: child_hashes<TPC, PCA_OP_XOR>(ws, ra, rb, imm, T, lane, h, hf); break;
    case PCA_OP_SHL: child_hashes<TPC, PCA_OP_SHL>(ws, ra, rb, imm, T, lane, h, hf); break;
    case PCA_OP_SHR: child_hashes<TPC, PCA_OP_SHR>(ws, ra, rb, imm, T, lane, h, hf); break;
    case PCA_OP_ASR: child_hashes<TPC, PCA_OP_ASR>(ws, ra, rb, imm, T, lane, h, hf); break;
    case PCA_OP_LDI: child_hashes<TPC, PCA_OP_LDI>(ws, ra, rb, imm, T, lane, h, hf); break;
    default: child_hashes<TPC, PCA_OP_ADDI>(ws, ra, rb, imm, T, lane, h, hf); break;
    }
}

/* Exact compare of child A (lane jA's child of the warp's parent, its new
   column and flags in shared memory, micro-op uA) with child B (parent qB of
   the level in HBM + micro-op uB), the whole warp cooperating: lane t
   rebuilds test t of child B (every register, the flags) and __all_sync
   decides. The requesting lane has already checked the task and (when it is
   part of the key) the live mask. All lanes must call it. */
template <int TPC>
__device__ bool warp_child_equal(const LevelDev &P, const InsertState<TPC> &A, uint64_t qA, int T,
                                 int jA, uint32_t uA, uint64_t qB, uint32_t uB, int lane)
{
    const uint32_t rdA = UOP_RD(uA), rdB = UOP_RD(uB);
    bool ok = true;
    if (lane < T) {
        const uint32_t resA = A.colA[lane][jA];
        const uint32_t fA = (uint32_t)(A.flagsA[lane >> 4][jA] >> (4 * (lane & 15))) & 15u;
        if (qB == qA) {
            /* same parent (about a fifth of the duplicates): only the written
               columns and the flags can differ, and the parent is in shared
               memory */
            const uint32_t a2 = A.R[UOP_A(uB)][lane], b2 = A.R[UOP_B(uB)][lane];
            const uint32_t resB = pca_alu(UOP_OP(uB), a2, b2, UOP_IMM(uB));
            const uint32_t fB = pca_alu_flags(UOP_OP(uB), a2, b2, UOP_IMM(uB), resB, A.F[lane]);
            ok = fA == fB;
            if (rdA == rdB) {
                ok &= resA == resB;
            } else {
                ok &= resA == A.R[rdA][lane];   /* B keeps the parent's rdA column */
                ok &= resB == A.R[rdB][lane];   /* A keeps the parent's rdB column */
            }
        } else {
            const uint16_t *RB = P.regs + qB * 8 * TPC + lane;
            const uint32_t a2 = RB[UOP_A(uB) * TPC], b2 = RB[UOP_B(uB) * TPC];
            const uint32_t resB = pca_alu(UOP_OP(uB), a2, b2, UOP_IMM(uB));
            const uint32_t fB = pca_alu_flags(UOP_OP(uB), a2, b2, UOP_IMM(uB), resB,
                                              P.flags[qB * TPC + lane]);
            ok = fA == fB;
#pragma unroll
            for (uint32_t r = 1; r < 8; r++) {
                const uint32_t vA = r == rdA ? resA : (uint32_t)A.R[r][lane];
                const uint32_t vB = r == rdB ? resB : (uint32_t)RB[r * TPC];
                ok &= vA == vB;
            }
        }
    }
    return __all_sync(0xFFFFFFFFu, ok);
}

/* Six CTAs per SM (40 registers a thread, 26 KB of shared memory a CTA at
   32 tests): measured 3% faster than eight CTAs at 32 registers, whose
   spills cost more than the extra warps hide. */
template <int TPC>
__global__ void __launch_bounds__(kThreads, 6)
k_expand_insert(LevelDev P, TaskDev task, unsigned long long *table, uint64_t tmask,
                uint32_t *status, uint32_t split_log2, const uint32_t *fcr_up, uint32_t *next)
{
    __shared__ InsertState<TPC> sws[kWarpsPerBlock];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    InsertState<TPC> &ws = sws[wib];
    const uint32_t split = 1u << split_log2;
    /* a work item is a parent (split 1) or one of `split` slices of its
       chunk list: small levels spread each parent over several warps. Warps
       draw items from a counter (`next`, zero at launch; lane 0 fetches the
       next item while the warp works on the current one): a parent's cost
       (its children, their probes and exact compares) varies widely, and
       fixed shares left the first SMs idle for ~18% of the launch while the
       last finished (a warp stages its own parent, so no L1 sharing is lost;
       measured 1.59 -> 1.48 ms per solve). Items < 2^33 (levels below 2^28
       states, slices only for levels below 2^12). */
    const uint64_t items = P.n << split_log2;
    uint32_t nx = 0;
    if (lane == 0) nx = atomicAdd(next, 1u);
    for (uint64_t it = __shfl_sync(0xFFFFFFFFu, nx, 0); it < items;
         it = __shfl_sync(0xFFFFFFFFu, nx, 0)) {
        if (lane == 0) nx = atomicAdd(next, 1u);
        const uint64_t q = it >> split_log2;
        const uint32_t g = (uint32_t)it & (split - 1);
        const uint32_t tid = P.task[q];
        if (!task.active[tid]) continue;
        const int T = task.T[tid];
        __syncwarp();
        load_insert_state<TPC>(ws, P.regs, P.flags, q, lane);
        const uint32_t live = P.live[q];
        __syncwarp();
        if (lane >= 1 && lane < 8) ws.colh[lane] = col_final(lane, hash_column<TPC>(ws.R[lane]));
        __syncwarp();
        uint64_t regsum = task_final(tid);
#pragma unroll
        for (int r = 1; r < 8; r++) regsum += ws.colh[r];
        const uint32_t m = (live >> 1) & 127u;
        const uint32_t base = c_cand_off[m];
        const uint32_t k0 = c_chunk_off[m], k1 = c_chunk_off[m + 1];
        const uint32_t per = (k1 - k0 + split - 1) >> split_log2;
        const uint32_t ka = min(k1, k0 + g * per), kb = min(k1, ka + per);
        const uint32_t wdead = deadable_writes(P, fcr_up, q);
        const uint32_t wldi = fcr_up && (P.own[q] & 1u) ? P.rdl[q] : 0u;
        const bool twin_later = P.twin[q] != 0;
        for (uint32_t k = ka; k < kb; k++) {
            const uint32_t ch = c_chunks[k], start = ch >> 8, cnt = ch & 255u;
            bool valid = (uint32_t)lane < cnt;
            const uint32_t c = start + (valid ? lane : 0);
            const uint32_t u = c_cand_uop[base + c];
            const uint32_t op = UOP_OP(u), rd = UOP_RD(u);
            if ((wdead >> rd & 1u) && op != PCA_OP_LDI && !uop_reads(u, rd)) valid = false;
            if (ldi_swap(u, wldi)) valid = false;
            if (u >> 31) valid = false;   /* an earlier sibling's state (same value and flags) */
            if (twin_later && op != PCA_OP_LDI) valid = false;   /* k_twins */
            if (!__any_sync(0xFFFFFFFFu, valid)) continue;
            uint64_t h, hf;
            __syncwarp();   /* the previous chunk's compares are done with colA */
            child_hashes_any<TPC>(op, ws, UOP_A(u), UOP_B(u), UOP_IMM(u), T, lane, h, hf);
            __syncwarp();
            uint64_t H = regsum - ws.colh[rd] + col_final(rd, h) + hf;
            if (task.key_live) H += live_final(live | (1u << rd));
            const uint64_t ref = (q << 12) | c;
            const unsigned long long mine = ((H >> 40) << 40) | (ref + 1);
            uint64_t idx = H & tmask;
            uint32_t probes = 0;
            bool done = !valid;
            /* lanes probe in parallel; a tag match is settled by an exact
               warp-wide compare, one requesting lane at a time */
            while (__any_sync(0xFFFFFFFFu, !done)) {
                bool needcmp = false;
                unsigned long long s = 0;
                if (!done) {
                    s = *((volatile unsigned long long *)&table[idx]);
                    if (s == 0) {
                        const unsigned long long old = atomicCAS(&table[idx], 0ull, mine);
                        if (old == 0) done = true;
                        else s = old;
                    }
                    if (!done) needcmp = (s >> 40) == (mine >> 40);
                }
                /* a tag match first settles the stored child's task, live
                   mask and micro-op in its own lane (all lanes at once);
                   only a match on those takes a warp-wide compare */
                uint64_t qB = 0;
                uint32_t uB = 0;
                if (needcmp) {
                    const uint64_t oref = (s & kRefMask) - 1;
                    qB = oref >> 12;
                    uint32_t liveB = live;
                    if (qB != q) {
                        const uint32_t tB = P.task[qB];
                        liveB = P.live[qB];
                        needcmp = tB == tid;
                    }
                    uB = c_cand_uop[c_cand_off[(liveB >> 1) & 127u] + (uint32_t)(oref & 4095)];
                    if (task.key_live && (live | (1u << rd)) != (liveB | (1u << UOP_RD(uB))))
                        needcmp = false;
                }
                uint32_t req = __ballot_sync(0xFFFFFFFFu, needcmp);
                bool eq = false;
                while (req) {
                    const int j = __ffs(req) - 1;
                    req &= req - 1;
                    const uint32_t uj = __shfl_sync(0xFFFFFFFFu, u, j);
                    const uint32_t ubj = __shfl_sync(0xFFFFFFFFu, uB, j);
                    const uint64_t qbj = __shfl_sync(0xFFFFFFFFu, qB, j);
                    const bool e = warp_child_equal<TPC>(P, ws, q, T, j, uj, qbj, ubj, lane);
                    if (lane == j) eq = e;
                }
                if (!done) {
                    if (needcmp && eq) {
                        /* same state: keep the smaller ref (the DFS-first child) */
                        uint64_t oref = (s & kRefMask) - 1;
                        while (ref < oref) {
                            const unsigned long long old = atomicCAS(&table[idx], s, mine);
                            if (old == s) break;
                            s = old;
                            oref = (s & kRefMask) - 1;
                        }
                        done = true;
                    } else {
                        idx = (idx + 1) & tmask;
                        if (++probes >= kMaxProbes) {
                            atomicOr(status, kStatusTableFull);
                            done = true;
                        }
                    }
                }
            }
        }
    }
}

/* Flag twins. Two states of a level with the same registers, live mask and
   task but different flags (e.g. two independent instructions in either
   order, or two ops that write the same value with different flags) have,
   for every flag-setting candidate c (every op but LDI), children that are
   the same state under either pruning key: the same registers, c's flags
   and the same live mask; and c has the same index in both parents' lists
   (the lists depend on live only). The earlier state's child is the smaller
   ref, so no flag-setting child of a later twin is ever the DFS-first
   representative: k_twins marks the later twins (twin[q] = 1) and the insert
   kernel skips those children. One warp per state (lane = test): a hash of
   r1..r7, live and task, then an open-addressed table whose slot keeps the
   class's lowest rank, every tag match settled by an exact warp-wide
   compare. Probing is bounded (kStatusTableFull). twin[] is zeroed
   beforehand. */
template <int TPC>
__global__ void k_twins(LevelDev P, TaskDev task, unsigned long long *table, uint64_t tmask,
                        uint8_t *twin, uint32_t *status)
{
    const int lane = threadIdx.x & 31;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t q = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < P.n; q += nw) {
        const uint32_t tid = P.task[q];
        if (!task.active[tid]) continue;
        const uint32_t live = P.live[q];
        uint32_t col[7];
        uint64_t h = 0;
        if (lane < TPC) {
            const uint16_t *src = P.regs + q * 8 * TPC + lane;
            uint64_t w = 0x243F6A8885A308D3ull ^ (uint64_t)lane;
#pragma unroll
            for (int r = 1; r < 8; r++) {
                col[r - 1] = src[r * TPC];
                w = chain(w, col[r - 1]);
            }
            h = fmix64(w);
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) h += __shfl_xor_sync(0xFFFFFFFFu, h, o);
        const uint64_t H = h + live_final(live) + task_final(tid);
        const unsigned long long mine = ((H >> 40) << 40) | (q + 1);
        uint64_t idx = H & tmask;
        uint32_t probes = 0;
        for (;;) {
            unsigned long long s = 0;
            if (lane == 0) {
                s = *((volatile unsigned long long *)&table[idx]);
                if (s == 0) s = atomicCAS(&table[idx], 0ull, mine);
            }
            s = __shfl_sync(0xFFFFFFFFu, s, 0);
            if (s == 0) break;   /* the first of its class so far */
            bool eq = false;
            if ((s >> 40) == (mine >> 40)) {
                const uint64_t qB = (s & kRefMask) - 1;
                eq = P.task[qB] == tid && P.live[qB] == live;
                if (eq) {
                    bool ok = true;
                    if (lane < TPC) {
                        const uint16_t *srcB = P.regs + qB * 8 * TPC + lane;
#pragma unroll
                        for (int r = 1; r < 8; r++) ok &= srcB[r * TPC] == col[r - 1];
                    }
                    eq = __all_sync(0xFFFFFFFFu, ok);
                }
            }
            if (eq) {
                /* one class: the slot keeps the lowest rank, every other
                   member is marked */
                if (lane == 0) {
                    unsigned long long cur = s;
                    for (;;) {
                        const uint64_t m = (cur & kRefMask) - 1;
                        if (q > m) { twin[q] = 1; break; }
                        const unsigned long long old = atomicCAS(&table[idx], cur, mine);
                        if (old == cur) { twin[m] = 1; break; }
                        cur = old;
                    }
                }
                break;
            }
            idx = (idx + 1) & tmask;
            if (++probes >= kMaxProbes) {
                if (lane == 0) atomicOr(status, kStatusTableFull);
                break;
            }
        }
    }
}

/* Mark each table winner in the child bitmap; count them. A thread reads
   four slots (two 16-byte loads, both issued before either is used) per
   step: the table is larger than L2 and its scan is the kernel's traffic.
   slots is a power of two >= 1024 and the table 16-byte aligned. */
__device__ __forceinline__ uint32_t mark_slot(unsigned long long s, const uint64_t *child_off,
                                              uint32_t *bitmap)
{
    if (!s) return 0;
    const uint64_t ref = (s & kRefMask) - 1;
    const uint64_t L = child_off[ref >> 12] + (ref & 4095);
    atomicOr(&bitmap[L >> 5], 1u << (L & 31));
    return 1;
}

__global__ void k_mark(const unsigned long long *table, uint64_t slots, const uint64_t *child_off,
                       uint32_t *bitmap, unsigned long long *count)
{
    const ulonglong2 *t2 = reinterpret_cast<const ulonglong2 *>(table);
    const uint64_t quads = slots / 4;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint32_t local = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < quads; i += stride) {
        const ulonglong2 a = t2[2 * i], b = t2[2 * i + 1];
        local += mark_slot(a.x, child_off, bitmap) + mark_slot(a.y, child_off, bitmap) +
                 mark_slot(b.x, child_off, bitmap) + mark_slot(b.y, child_off, bitmap);
    }
    for (int o = 16; o; o >>= 1) local += __shfl_down_sync(0xFFFFFFFFu, local, o);
    if ((threadIdx.x & 31) == 0 && local) atomicAdd(count, (unsigned long long)local);
}

/* Keep every child (no pruning): set all bits below `total`. */
__global__ void k_mark_all(uint32_t *bitmap, uint64_t words, uint64_t total)
{
    for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w < words;
         w += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t lo = w * 32;
        uint32_t v = 0xFFFFFFFFu;
        if (lo + 32 > total) v = total > lo ? (uint32_t)((1ull << (total - lo)) - 1) : 0u;
        bitmap[w] = v;
    }
}

__global__ void k_popc(const uint32_t *bitmap, uint64_t words, uint64_t *cnt)
{
    for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w < words;
         w += (uint64_t)gridDim.x * blockDim.x)
        cnt[w] = __popc(bitmap[w]);
}

/* child_off[i] = number of candidates of state i, 0 when its task is not
   searched any more (scanned afterwards). */
__global__ void k_child_counts(const uint8_t *live, const uint16_t *task, const uint8_t *active,
                               uint64_t n, uint64_t *cnt)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t m = (live[i] >> 1) & 127u;
        cnt[i] = active[task[i]] ? c_cand_off[m + 1] - c_cand_off[m] : 0;
    }
}

/* One warp's shared memory in the materialisation: the parent's register
   block in the level's own layout (8 columns of TPC tests) and the current
   child's new column and flags, from which each lane writes one 16-byte
   piece of the child. */
template <int TPC>
struct MatState {
    __align__(16) uint16_t PR[8 * TPC];
    __align__(16) uint16_t CB[TPC];
    __align__(16) uint8_t FB[TPC];
};

/* Write the marked children of each parent, in rank (DFS) order. A child's
   register block (8 x TPC halves) is written as TPC 16-byte pieces, one per
   lane, and its flags as TPC/16 pieces: lane t first computes the new value
   and flags of test t into shared memory, then lane L copies piece L from
   the parent's block, or from the new column when the piece lies in the
   written register's column. Level blocks start on 256-byte boundaries (the
   arena's allocation unit) and a state's block is 256 or 512 bytes, so
   every piece is 16-byte aligned. */
template <int TPC>
__global__ void __launch_bounds__(kThreads)
k_materialize(LevelDev P, TaskDev task, const uint32_t *bitmap, const uint64_t *word_off,
              LevelOut C, uint32_t split_log2, uint32_t *fcr, const uint32_t *fcr_up)
{
    static_assert(TPC == 16 || TPC == 32, "a state holds 16 or 32 tests");
    constexpr int kPieces = 8 * TPC * 2 / 16;   /* = TPC: lanes 0..TPC-1 */
    constexpr int kFlagPieces = TPC / 16;
    constexpr int kPiecesPerCol = TPC / 8;
    __shared__ MatState<TPC> sms[kWarpsPerBlock];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    MatState<TPC> &ms = sms[wib];
    const uint32_t my_col = (uint32_t)lane / kPiecesPerCol;   /* column of piece `lane` */
    const uint4 *my_new = reinterpret_cast<const uint4 *>(ms.CB) + lane % kPiecesPerCol;
    const uint4 *my_old = reinterpret_cast<const uint4 *>(ms.PR) + lane;
    const uint64_t nw = (uint64_t)gridDim.x * kWarpsPerBlock;
    const uint32_t split = 1u << split_log2;
    /* work items as in k_expand_insert: a parent, or a slice of its
       32-candidate groups */
    for (uint64_t it = (uint64_t)blockIdx.x * kWarpsPerBlock + wib; it < (P.n << split_log2);
         it += nw) {
        const uint64_t q = it >> split_log2;
        const uint32_t g = (uint32_t)it & (split - 1);
        const uint32_t tid = P.task[q];
        if (!task.active[tid]) continue;
        const int T = task.T[tid];
        __syncwarp();
        if (lane < kPieces)
            reinterpret_cast<uint4 *>(ms.PR)[lane] =
                reinterpret_cast<const uint4 *>(P.regs + q * 8 * TPC)[lane];
        const uint32_t pf = lane < TPC ? P.flags[q * TPC + lane] : 0u;
        const uint32_t live = P.live[q];
        __syncwarp();
        const uint32_t m = (live >> 1) & 127u;
        const uint32_t base = c_cand_off[m], nc = c_cand_off[m + 1] - base;
        const uint64_t off = P.child_off[q];
        const uint32_t W = deadable_writes(P, fcr_up, q);
        const uint32_t groups = (nc + 31) >> 5;
        const uint32_t per = (groups + split - 1) >> split_log2;
        const uint32_t ga = min(groups, g * per), gb = min(groups, ga + per);
        for (uint32_t c0 = ga * 32; c0 < gb * 32; c0 += 32) {
            /* each lane settles its own candidate (kept?, rank, micro-op and
               the child's links) so the per-child loop below needs no
               global load */
            const uint32_t c = c0 + lane;
            bool keep = false;
            uint64_t rank = 0;
            uint32_t u = 0;
            if (c < nc) {
                const uint64_t L = off + c;
                const uint32_t wv = bitmap[L >> 5];
                keep = (wv >> (L & 31)) & 1u;
                if (keep) {
                    rank = word_off[L >> 5] + __popc(wv & ((1u << (L & 31)) - 1u));
                    u = c_cand_uop[base + c];
                    C.live[rank] = (uint8_t)(live | (1u << UOP_RD(u)));
                    C.rdl[rank] = (uint8_t)UOP_RD(u);
                    C.task[rank] = (uint16_t)tid;
                    C.parent[rank] = (uint32_t)q;
                    C.cidx[rank] = (uint16_t)c;
                    /* a write read by u is used; the one u overwrites is gone */
                    C.own[rank] = (uint8_t)((W & ~((1u << UOP_A(u)) | (1u << UOP_B(u)) |
                                                   (1u << UOP_RD(u))) & 0xFEu) |
                                            (UOP_OP(u) == PCA_OP_LDI ? 1u : 0u));
                    /* first kept child of q per written register */
                    if (fcr) atomicMin(&fcr[q * 8 + UOP_RD(u)], (uint32_t)rank);
                }
            }
            uint32_t bal = __ballot_sync(0xFFFFFFFFu, keep);
            while (bal) {
                const int j = __ffs(bal) - 1;
                bal &= bal - 1;
                const uint64_t rk = __shfl_sync(0xFFFFFFFFu, rank, j);
                const uint32_t uj = __shfl_sync(0xFFFFFFFFu, u, j);
                const uint32_t op = UOP_OP(uj), rd = UOP_RD(uj);
                if (lane < TPC) {
                    const uint32_t a = ms.PR[UOP_A(uj) * TPC + lane];
                    const uint32_t b = ms.PR[UOP_B(uj) * TPC + lane];
                    uint32_t res = pca_alu(op, a, b, UOP_IMM(uj));
                    uint32_t f = pca_alu_flags(op, a, b, UOP_IMM(uj), res, pf);
                    if (lane >= T) { res = 0; f = 0; }
                    ms.CB[lane] = (uint16_t)res;
                    ms.FB[lane] = (uint8_t)f;
                }
                __syncwarp();
                if (lane < kPieces) {
                    const uint4 pv = *(my_col == rd ? my_new : my_old);
                    reinterpret_cast<uint4 *>(C.regs + rk * 8 * TPC)[lane] = pv;
                    /* the lane holding tests 0..7 of a column also writes
                       tests 0..3 of it into the probe (8 lanes, 64 bytes) */
                    if (lane % kPiecesPerCol == 0)
                        reinterpret_cast<uint2 *>(C.probe + rk * 32)[my_col] = make_uint2(pv.x, pv.y);
                }
                if (lane < kFlagPieces)
                    reinterpret_cast<uint4 *>(C.flags + rk * TPC)[lane] =
                        reinterpret_cast<const uint4 *>(ms.FB)[lane];
                __syncwarp();
            }
        }
    }
}

/* The lean form of k_materialize, for a level that only the last position
 * reads (the lane-per-prefix scan: each state's 64-byte probe, its links,
 * and on a hit the registers that k_suffix_lanes recomputes from the
 * parent). Per kept child it writes live, rdl, task, parent, cidx, own and
 * the probe, computed from the parent's probe: no register block and no
 * flags, 64 bytes a state instead of 8 x TPC x 2 + TPC + 64. A warp takes a
 * parent (or a slice of its 32-candidate groups, as k_materialize), stages
 * the parent's probe in shared memory, and each lane settles its own
 * candidate. */
template <int TPC>
__global__ void __launch_bounds__(kThreads)
k_materialize_probe(LevelDev P, TaskDev task, const uint32_t *bitmap, const uint64_t *word_off,
                    LevelOut C, uint32_t split_log2, const uint32_t *fcr_up, uint32_t *next)
{
    static_assert(TPC == 16 || TPC == 32, "a state holds 16 or 32 tests");
    __shared__ __align__(16) uint16_t spp[kWarpsPerBlock][8][4];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    uint16_t (&PP)[8][4] = spp[wib];
    const uint32_t split = 1u << split_log2;
    /* work items drawn from a counter, as in k_expand_insert (measured
       0.03 ms faster per solve than fixed shares) */
    const uint64_t items = P.n << split_log2;
    uint32_t nx = 0;
    if (lane == 0) nx = atomicAdd(next, 1u);
    for (uint64_t it = __shfl_sync(0xFFFFFFFFu, nx, 0); it < items;
         it = __shfl_sync(0xFFFFFFFFu, nx, 0)) {
        if (lane == 0) nx = atomicAdd(next, 1u);
        const uint64_t q = it >> split_log2;
        const uint32_t g = (uint32_t)it & (split - 1);
        const uint32_t tid = P.task[q];
        if (!task.active[tid]) continue;
        const int T = task.T[tid];
        __syncwarp();
        if (lane < 8)
            reinterpret_cast<uint2 *>(&PP[0][0])[lane] =
                reinterpret_cast<const uint2 *>(P.probe + q * 32)[lane];
        const uint32_t live = P.live[q];
        __syncwarp();
        const uint32_t m = (live >> 1) & 127u;
        const uint32_t base = c_cand_off[m], nc = c_cand_off[m + 1] - base;
        const uint64_t off = P.child_off[q];
        const uint32_t W = deadable_writes(P, fcr_up, q);
        const uint32_t groups = (nc + 31) >> 5;
        const uint32_t per = (groups + split - 1) >> split_log2;
        const uint32_t ga = min(groups, g * per), gb = min(groups, ga + per);
        for (uint32_t c = ga * 32 + lane; c < gb * 32; c += 32) {
            if (c >= nc) continue;
            const uint64_t L = off + c;
            const uint32_t wv = bitmap[L >> 5];
            if (!((wv >> (L & 31)) & 1u)) continue;
            const uint64_t rank = word_off[L >> 5] + __popc(wv & ((1u << (L & 31)) - 1u));
            const uint32_t u = c_cand_uop[base + c];
            const uint32_t rd = UOP_RD(u), ra = UOP_A(u), rb = UOP_B(u);
            C.live[rank] = (uint8_t)(live | (1u << rd));
            C.rdl[rank] = (uint8_t)rd;
            C.task[rank] = (uint16_t)tid;
            C.parent[rank] = (uint32_t)q;
            C.cidx[rank] = (uint16_t)c;
            C.own[rank] = (uint8_t)((W & ~((1u << ra) | (1u << rb) | (1u << rd)) & 0xFEu) |
                                    (UOP_OP(u) == PCA_OP_LDI ? 1u : 0u));
            /* the written register on tests 0..3 (0 past the task's tests,
               as k_materialize writes them) */
            uint32_t nv[4];
#pragma unroll
            for (int t = 0; t < 4; t++)
                nv[t] = t < T ? pca_alu(UOP_OP(u), PP[ra][t], PP[rb][t], UOP_IMM(u)) & 0xFFFFu
                              : 0u;
            const uint32_t lo = nv[0] | (nv[1] << 16), hi = nv[2] | (nv[3] << 16);
            uint4 *dst = reinterpret_cast<uint4 *>(C.probe + rank * 32);
#pragma unroll
            for (int h = 0; h < 4; h++) {
                const uint4 old = reinterpret_cast<const uint4 *>(&PP[0][0])[h];
                uint4 v = old;
                if (rd == 2u * h) { v.x = lo; v.y = hi; }
                if (rd == 2u * h + 1) { v.z = lo; v.w = hi; }
                dst[h] = v;
            }
        }
    }
}

/* hist[task][mask] += states of that task with that liveness mask. Lanes
   with the same key are counted by one atomic (states of a level are
   grouped by task and mostly by mask). With n_dev set, the level holds
   min(n, *n_dev) states (n is then the space written, an upper bound). */
__global__ void k_task_hist(const uint8_t *live, const uint16_t *task, uint64_t n,
                            const unsigned long long *n_dev, unsigned long long *hist)
{
    if (n_dev && *n_dev < n) n = *n_dev;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t n_round = (n + 31) & ~31ull;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_round; i += stride) {
        const bool valid = i < n;
        const uint32_t key = valid ? (uint32_t)task[i] * 128u + ((live[i] >> 1) & 127u) : ~0u;
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, key);
        if (valid && (threadIdx.x & 31) == __ffs(peers) - 1)
            atomicAdd(&hist[key], (unsigned long long)__popc(peers));
    }
}

/* The same with a per-block histogram in shared memory (nbins u32 counters,
   nbins = tasks x 128 <= 4096), flushed with one global atomic per nonzero
   bin: a level's states crowd a few bins, and per-warp global atomics on
   them serialize. */
__global__ void k_task_hist_smem(const uint8_t *live, const uint16_t *task, uint64_t n,
                                 const unsigned long long *n_dev, uint32_t nbins,
                                 unsigned long long *hist)
{
    extern __shared__ uint32_t sh_hist[];
    if (n_dev && *n_dev < n) n = *n_dev;
    for (uint32_t b = threadIdx.x; b < nbins; b += blockDim.x) sh_hist[b] = 0;
    __syncthreads();
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t n_round = (n + 31) & ~31ull;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_round; i += stride) {
        const bool valid = i < n;
        const uint32_t key = valid ? (uint32_t)task[i] * 128u + ((live[i] >> 1) & 127u) : ~0u;
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, key);
        if (valid && (threadIdx.x & 31) == __ffs(peers) - 1 && key < nbins)
            atomicAdd(&sh_hist[key], (uint32_t)__popc(peers));
    }
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < nbins; b += blockDim.x)
        if (sh_hist[b]) atomicAdd(&hist[b], (unsigned long long)sh_hist[b]);
}

/* ---- solutions ----------------------------------------------------------- */

struct SolBuf {
    unsigned long long *count;    /* solving (prefix, mids, class) records */
    ulonglong2 *rec;              /* x = prefix rank, y = m1<<32 | m2<<16 | class */
    uint64_t cap;
    unsigned long long *first;    /* atomicMin of a packed DFS-order key */
    unsigned long long *evals;    /* value-class evaluations the suffix kernels ran
                                     (each class of an operand pair counts one) */
};

/* Adds a warp's per-lane evaluation counts to S.evals (all lanes call it). */
__device__ __forceinline__ void flush_evals(const SolBuf &S, unsigned long long nev, int lane)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) nev += __shfl_down_sync(0xFFFFFFFFu, nev, o);
    if (lane == 0 && nev) atomicAdd(S.evals, nev);
}

__device__ __forceinline__ void record_solution(const SolBuf &S, uint64_t q, uint32_t m1,
                                                uint32_t m2, uint32_t vc, uint32_t first_c)
{
    unsigned long long slot = atomicAdd(S.count, 1ull);
    if (slot < S.cap)
        S.rec[slot] = make_ulonglong2(q, ((unsigned long long)m1 << 32) | (m2 << 16) | vc);
    unsigned long long key = ((unsigned long long)(q & 0xFFFFFFFull) << 36) |
                             ((unsigned long long)m1 << 24) | ((unsigned long long)m2 << 12) |
                             first_c;
    atomicMin(S.first, key);
}

/* Leaf check of a materialized level (count mode): state q solves through
 * live register r when regs[q][r][t] == target[t] for every test. */
template <int TPC>
__global__ void k_leaf(LevelDev P, TaskDev task, SolBuf S)
{
    const int lane = threadIdx.x & 31;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t q = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < P.n; q += nw) {
        const uint32_t tid = P.task[q];
        if (!task.active[tid]) continue;
        const int T = task.T[tid];
        const uint32_t tgt = lane < T ? task.target[tid * 32 + lane] : 0u;
        const uint32_t live = P.live[q];
        for (uint32_t r = 1; r < 8; r++) {
            if (!((live >> r) & 1u)) continue;
            bool ok = lane >= T || P.regs[q * 8 * TPC + r * TPC + lane] == tgt;
            if (__all_sync(0xFFFFFFFFu, ok) && lane == 0) record_solution(S, q, 0, 0, r, r);
        }
    }
}

/* Which of the ops of an operand-pair entry give t from (x, y): bit k < 9
   for the ALU op kPairOps[k], bit 9 for x + e (an ADDI, e its immediate
   sign-extended to 16 bits). Every op is evaluated, with no branch. */
__device__ __forceinline__ uint32_t pair_hits(uint32_t x, uint32_t y, uint32_t e, uint32_t t)
{
    const uint32_t s = y & 15u;
    uint32_t h = 0;
    h |= (uint32_t)(((x + y) & 0xFFFFu) == t);
    h |= (uint32_t)(((x - y) & 0xFFFFu) == t) << 1;
    h |= (uint32_t)(((x * y) & 0xFFFFu) == t) << 2;
    h |= (uint32_t)((x & y) == t) << 3;
    h |= (uint32_t)((x | y) == t) << 4;
    h |= (uint32_t)((x ^ y) == t) << 5;
    h |= (uint32_t)(((x << s) & 0xFFFFu) == t) << 6;
    h |= (uint32_t)((x >> s) == t) << 7;
    h |= (uint32_t)((uint32_t)(uint16_t)((int16_t)(uint16_t)x >> s) == t) << 8;
    h |= (uint32_t)(((x + e) & 0xFFFFu) == t) << 9;
    return h;
}

__device__ __forceinline__ uint32_t pair_op(uint32_t k)
{
    switch (k) {
    case 0: return PCA_OP_ADD;
    case 1: return PCA_OP_SUB;
    case 2: return PCA_OP_MUL;
    case 3: return PCA_OP_AND;
    case 4: return PCA_OP_OR;
    case 5: return PCA_OP_XOR;
    case 6: return PCA_OP_SHL;
    case 7: return PCA_OP_SHR;
    case 8: return PCA_OP_ASR;
    default: return PCA_OP_ADDI;
    }
}

/* Scan the value classes of mask m against the warp's state, with operand
 * registers remapped: a register equal to rd2 reads spare column 9, else a
 * register equal to rd1 reads column 8 (rd = 8 means "none").
 *
 * need1 / need2 (0 = none): registers the last instruction must read. At a
 * depth K reached only after depth K-1 was searched without a solution,
 * every instruction of a solving program feeds a later one: an instruction
 * whose value nothing reads could be dropped, leaving a solving program of
 * K-1 instructions in the same candidate space. So the last instruction
 * reads the register the one before it wrote (need1), and need2 names an
 * earlier write nothing else read. Only classes that read need1 are
 * scanned, from the per-register class lists; the solutions are the same. */
template <int TPC, int FT>
__device__ __forceinline__ void scan_last(const WarpState<TPC> &ws, int T,
                                          uint32_t m, uint32_t rd1, uint32_t rd2, uint32_t tgt,
                                          uint32_t tgt0, uint32_t tgt1, uint32_t tgt2, int lane,
                                          const SolBuf &S, uint64_t q, uint32_t m1, uint32_t m2,
                                          uint32_t need1, uint32_t need2, unsigned long long &nev)
{
    const uint32_t vbase = c_vc_off[m];
    if (need1) {
        /* the classes reading need1, one operand pair (or ADDI) per lane,
           every op of the pair evaluated on the first two tests at once */
        const uint32_t p0 = c_pr_off[m * 8 + need1], np = c_pr_off[m * 8 + need1 + 1] - p0;
        if (!need2 && lane == 0) nev += c_pr_ev[m * 8 + need1];
        for (uint32_t b0 = 0; b0 < np; b0 += 32) {
            const uint32_t i = b0 + lane;
            uint32_t hits = 0, ra = 0, rb = 0, e = 0;
            if (i < np) {
                const uint32_t d = c_pr[p0 + i];
                const uint32_t a = d & 7u, b = (d >> 3) & 7u;
                if (!need2 || a == need2 || b == need2) {
                    if (need2) nev += __popc((d >> 6) & 0x3FFu);
                    ra = a == rd2 ? 9u : a == rd1 ? 8u : a;
                    rb = b == rd2 ? 9u : b == rd1 ? 8u : b;
                    e = (uint32_t)(uint16_t)(int16_t)(int8_t)(uint8_t)(d >> 16);
                    hits = pair_hits(ws.R[ra][0], ws.R[rb][0], e, tgt0) & (d >> 6) & 0x3FFu;
                    if (FT >= 2 && T >= 2 && hits)
                        hits &= pair_hits(ws.R[ra][1], ws.R[rb][1], e, tgt1);
                    if (FT >= 3 && T >= 3 && hits)
                        hits &= pair_hits(ws.R[ra][2], ws.R[rb][2], e, tgt2);
                }
            }
            uint32_t bal = __ballot_sync(0xFFFFFFFFu, hits != 0);
            while (bal) {
                const int j = __ffs(bal) - 1;
                bal &= bal - 1;
                uint32_t hj = __shfl_sync(0xFFFFFFFFu, hits, j);
                const uint32_t aj = __shfl_sync(0xFFFFFFFFu, ra, j);
                const uint32_t bj = __shfl_sync(0xFFFFFFFFu, rb, j);
                const uint32_t ej = __shfl_sync(0xFFFFFFFFu, e, j);
                while (hj) {
                    const uint32_t k = (uint32_t)(__ffs(hj) - 1);
                    hj &= hj - 1;
                    bool ok = true;
                    if (lane < T) {
                        const uint32_t x = ws.R[aj][lane], y = ws.R[bj][lane];
                        ok = (k == 9 ? ((x + ej) & 0xFFFFu) : pca_alu(pair_op(k), x, y, 0)) == tgt;
                    }
                    if (__all_sync(0xFFFFFFFFu, ok) && lane == 0) {
                        const uint32_t cj = c_pr_cls[(uint64_t)(p0 + b0 + j) * 10 + k];
                        record_solution(S, q, m1, m2, cj, c_vc_first[vbase + cj]);
                    }
                }
            }
        }
        return;
    }
    const uint32_t *uops = c_vc_uop + vbase;
    const uint16_t *list = nullptr;
    const uint32_t nvc = c_vc_off[m + 1] - vbase;
    for (uint32_t b0 = 0; b0 < nvc; b0 += 32) {
        const uint32_t i = b0 + lane;
        uint32_t u = 0;
        bool pass = false;
        if (i < nvc) {
            /* the first FT tests per lane; survivors are checked on all tests below */
            u = uops[i];
            uint32_t ra = UOP_A(u), rb = UOP_B(u);
            const bool reads2 = !need2 || ra == need2 || rb == need2;
            ra = ra == rd2 ? 9u : ra == rd1 ? 8u : ra;
            rb = rb == rd2 ? 9u : rb == rd1 ? 8u : rb;
            const uint32_t op = UOP_OP(u), imm = UOP_IMM(u);
            nev += reads2 ? 1u : 0u;
            pass = reads2 && pca_alu(op, ws.R[ra][0], ws.R[rb][0], imm) == tgt0 &&
                   (FT < 2 || T < 2 || pca_alu(op, ws.R[ra][1], ws.R[rb][1], imm) == tgt1) &&
                   (FT < 3 || T < 3 || pca_alu(op, ws.R[ra][2], ws.R[rb][2], imm) == tgt2);
        }
        uint32_t bal = __ballot_sync(0xFFFFFFFFu, pass);
        while (bal) {
            const int j = __ffs(bal) - 1;
            bal &= bal - 1;
            const uint32_t uj = __shfl_sync(0xFFFFFFFFu, u, j);
            uint32_t ra = UOP_A(uj), rb = UOP_B(uj);
            ra = ra == rd2 ? 9u : ra == rd1 ? 8u : ra;
            rb = rb == rd2 ? 9u : rb == rd1 ? 8u : rb;
            bool ok = true;
            if (lane < T) ok = pca_alu(UOP_OP(uj), ws.R[ra][lane], ws.R[rb][lane], UOP_IMM(uj)) == tgt;
            if (__all_sync(0xFFFFFFFFu, ok) && lane == 0) {
                const uint32_t cj = list ? (uint32_t)list[b0 + j] : b0 + j;
                record_solution(S, q, m1, m2, cj, c_vc_first[vbase + cj]);
            }
        }
    }
}

/* The suffix kernels' view of a prefix: only its live columns (no operand
   of a candidate reads anything else; column 0 is zeroed once per warp)
   and no flags (no branchless op reads them). */
template <int TPC>
__device__ __forceinline__ void load_live_cols(WarpState<TPC> &ws, const uint16_t *regs,
                                               uint64_t q, uint32_t live, int lane)
{
    if (lane < TPC) {
        const uint16_t *src = regs + q * 8 * TPC + lane;
#pragma unroll
        for (int r = 1; r < 8; r++)
            if ((live >> r) & 1u) ws.R[r][lane] = src[r * TPC];
    }
}

/* A contiguous range of prefixes, optionally through a permutation: the
 * suffix kernel visits prefixes order[begin .. begin + count) (or begin ..
 * begin + count when order is null). */
/* Counts entries of order[0..n) that are >= n or repeat an earlier value
 * (seen: zeroed bitmap of n bits). Zero means order is a permutation. */
__global__ void k_check_perm(const uint32_t *order, uint64_t n, uint32_t *seen,
                             unsigned long long *bad)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t v = order[i];
        if (v >= n) {
            atomicAdd(bad, 1ull);
            continue;
        }
        const uint32_t bit = 1u << (v & 31);
        if (atomicOr(&seen[v >> 5], bit) & bit) atomicAdd(bad, 1ull);
    }
}

struct PrefixRange {
    const uint32_t *order;
    uint64_t begin, count;
};

/* Suffix enumeration of depth SD (1..3) from the prefixes of level P in
 * range R whose task is active. Work item = (prefix, chunk of first-suffix
 * candidates); for SD = 1 the chunk is the whole prefix. Five CTAs per SM
 * (48 registers) measured fastest: at SD = 1 four CTAs at 64 registers hide
 * less latency and six spill the prefetched columns; at SD = 2 five CTAs
 * instead of the four that 56 registers allow cut a two-input depth-4
 * stage from 39 to 30 ms. */
template <int TPC, int SD, int FT>
__global__ void __launch_bounds__(kThreads, 5)
k_suffix(LevelDev P, TaskDev task, SolBuf S, uint32_t chunks_per_prefix, uint32_t chunk,
         PrefixRange R)
{
    __shared__ WarpState<TPC> sws[kWarpsPerBlock];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    WarpState<TPC> &ws = sws[wib];
    const uint64_t nw = (uint64_t)gridDim.x * kWarpsPerBlock;
    const uint64_t items = R.count * chunks_per_prefix;
    uint64_t loaded = ~0ull;
    uint32_t cur_task = ~0u, tgt = 0, tgt0 = 0, tgt1 = 0, tgt2 = 0;
    int T = 0;
    unsigned long long nev = 0;
    if (lane < TPC) ws.R[0][lane] = 0;
    bool cur_active = false;
    if constexpr (SD == 1) {
        /* one prefix per item, software-pipelined: the next prefix's
           links and columns are loaded while this one's classes are scanned
           (the scan is short, and waiting on those loads bounded the loop) */
        uint64_t nq = ~0ull;
        uint32_t ntid = 0, nlive = 0, nw0 = 0, ncol[7];
        auto fetch = [&](uint64_t i) {
            nq = ~0ull;
            if (i >= items) return;
            const uint64_t q = R.order ? (uint64_t)R.order[R.begin + i] : R.begin + i;
            if (q >= P.n) return;  /* orders are checked on the host; never index outside */
            nq = q;
            ntid = P.task[q];
            nlive = P.live[q];
            nw0 = P.rdl[q];
            const uint16_t *src = P.regs + q * 8 * TPC + (lane < TPC ? lane : 0);
#pragma unroll
            for (int r = 1; r < 8; r++) ncol[r - 1] = src[r * TPC];
        };
        uint64_t it = (uint64_t)blockIdx.x * kWarpsPerBlock + wib;
        fetch(it);
        for (; it < items; it += nw) {
            const uint64_t q = nq;
            const uint32_t tid = ntid, live = nlive, w0 = nw0;
            if (q != ~0ull) {
                __syncwarp();
                if (lane < TPC) {
#pragma unroll
                    for (int r = 1; r < 8; r++) ws.R[r][lane] = ncol[r - 1];
                }
                __syncwarp();
            }
            fetch(it + nw);
            if (q == ~0ull) continue;
            if (tid != cur_task) {
                cur_task = tid;
                cur_active = task.active[tid] != 0;
                T = task.T[tid];
                tgt = lane < T ? task.target[tid * 32 + lane] : 0u;
                tgt0 = task.target[tid * 32];
                tgt1 = task.target[tid * 32 + 1];
                if (FT >= 3) tgt2 = task.target[tid * 32 + 2];
            }
            if (!cur_active) continue;
            /* w0: the prefix's last write (0 at a root); some later
               instruction must read it (the rule scan_last states) */
            scan_last<TPC, FT>(ws, T, (live >> 1) & 127u, 8, 8, tgt, tgt0, tgt1, tgt2, lane, S, q, 0, 0, w0,
                           0, nev);
        }
        /* no flush: k_count_evals counts this depth's evaluations (nev is
           dead here and costs no register) */
        return;
    }
    for (uint64_t it = (uint64_t)blockIdx.x * kWarpsPerBlock + wib; it < items; it += nw) {
        const uint64_t qi = it / chunks_per_prefix;
        const uint32_t ck = (uint32_t)(it - qi * chunks_per_prefix);
        const uint64_t q = R.order ? (uint64_t)R.order[R.begin + qi] : R.begin + qi;
        if (q >= P.n) continue;  /* orders are checked on the host; never index outside */
        const uint32_t tid = P.task[q];
        if (tid != cur_task) {
            cur_task = tid;
            cur_active = task.active[tid] != 0;
            T = task.T[tid];
            tgt = lane < T ? task.target[tid * 32 + lane] : 0u;
            tgt0 = task.target[tid * 32];
            tgt1 = task.target[tid * 32 + 1];
            if (FT >= 3) tgt2 = task.target[tid * 32 + 2];
        }
        if (!cur_active) continue;
        const uint32_t live = P.live[q];
        if (q != loaded) {
            __syncwarp();
            load_live_cols<TPC>(ws, P.regs, q, live, lane);
            loaded = q;
            __syncwarp();
        }
        const uint32_t m0 = (live >> 1) & 127u;
        /* the prefix's last write (0 at a root): some later instruction
           must read it (the rule scan_last states) */
        const uint32_t w0 = P.rdl[q];
        const uint32_t cb0 = c_cand_off[m0], nc0 = c_cand_off[m0 + 1] - cb0;
        const uint32_t lo = ck * chunk, hi = min(nc0, lo + chunk);
        for (uint32_t i1 = lo; i1 < hi; i1++) {
            const uint32_t u1 = c_cand_uop[cb0 + i1];
            /* a middle writing the same value and flags as an earlier
               sibling leads to the states that sibling leads to: under OEP
               its subtree is the pruned duplicate (never the DFS-first) */
            if (task.dedup_mid && (u1 >> 31)) continue;
            const uint32_t rd1 = UOP_RD(u1);
            /* w0 still unread after u1: overwritten (dead, skip) or owed by
               a later instruction */
            const uint32_t owe0 = w0 && !uop_reads(u1, w0) ? w0 : 0u;
            if (owe0 && rd1 == owe0) continue;
            __syncwarp();
            if (lane < TPC)
                ws.R[8][lane] = lane < T ? pca_alu(UOP_OP(u1), ws.R[UOP_A(u1)][lane],
                                                   ws.R[UOP_B(u1)][lane], UOP_IMM(u1))
                                         : 0u;
            __syncwarp();
            const uint32_t m1 = (m0 | (1u << (rd1 - 1))) & 127u;
            if (SD == 2) {
                scan_last<TPC, FT>(ws, T, m1, rd1, 8, tgt, tgt0, tgt1, tgt2, lane, S, q, i1, 0, rd1, owe0,
                               nev);
                continue;
            }
            const uint32_t cb1 = c_cand_off[m1], nc1 = c_cand_off[m1 + 1] - cb1;
            for (uint32_t i2 = 0; i2 < nc1; i2++) {
                const uint32_t u2 = c_cand_uop[cb1 + i2];
                if (task.dedup_mid && (u2 >> 31)) continue;
                const uint32_t rd2 = UOP_RD(u2);
                /* writes still owed a read after u2 (u1's and maybe w0's);
                   one overwritten unread is dead, and the last instruction
                   reads rd2 and at most one more register */
                const uint32_t owe1 = uop_reads(u2, rd1) ? 0u : rd1;
                const uint32_t owe0b = owe0 && !uop_reads(u2, owe0) ? owe0 : 0u;
                if ((owe1 && rd2 == owe1) || (owe0b && rd2 == owe0b)) continue;
                if (owe1 && owe0b) continue;   /* three registers to read */
                const uint32_t need2 = owe1 ? owe1 : owe0b;
                uint32_t ra = UOP_A(u2), rb = UOP_B(u2);
                ra = ra == rd1 ? 8u : ra;
                rb = rb == rd1 ? 8u : rb;
                __syncwarp();
                if (lane < TPC)
                    ws.R[9][lane] = lane < T ? pca_alu(UOP_OP(u2), ws.R[ra][lane],
                                                       ws.R[rb][lane], UOP_IMM(u2))
                                             : 0u;
                __syncwarp();
                const uint32_t m2 = (m1 | (1u << (rd2 - 1))) & 127u;
                scan_last<TPC, FT>(ws, T, m2, rd2 == rd1 ? 8u : rd1, rd2, tgt, tgt0, tgt1, tgt2, lane, S,
                               q, i1, i2, rd2, need2, nev);
            }
        }
    }
    flush_evals(S, nev, lane);
}

/* The last position (suffix depth 1) with a lane per prefix: a warp takes
 * 32 prefixes of range R at once, each lane the operand pairs of its own
 * prefix that read the prefix's last write (the read rule, as scan_last),
 * every op of a pair evaluated on the first FT tests at once. A lane holds
 * nothing but its prefix's first FT test values of r0..r7 (in shared
 * memory, [test][register][lane], so lanes reading different registers hit
 * different banks) instead of the whole state: per prefix 7 sectors of the
 * level instead of seven 64-byte columns, and the warp's instructions are
 * not repeated for every prefix. A pair that passes the first FT tests is
 * checked on every test by the whole warp (lane = test) straight from the
 * level and recorded as the warp-per-prefix kernel records it, so the
 * records are the same. Every prefix of a level past the root has a last
 * write (no candidate of the branchless set writes r0); root prefixes
 * (w0 = 0) are left to k_suffix. */
template <int TPC, int FT>
__global__ void __launch_bounds__(kThreads, 5)
k_suffix_lanes(LevelDev P, TaskDev task, SolBuf S, PrefixRange R, LeanDev lean)
{
    __shared__ uint32_t sV[kWarpsPerBlock][FT][8][32];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    uint32_t (&V)[FT][8][32] = sV[wib];
#pragma unroll
    for (int t = 0; t < FT; t++) V[t][0][lane] = 0;
    const uint64_t nw = (uint64_t)gridDim.x * kWarpsPerBlock;
    uint32_t nev = 0;   /* this lane's prefixes' readable classes (the evaluation count) */
    for (uint64_t base = ((uint64_t)blockIdx.x * kWarpsPerBlock + wib) * 32; base < R.count;
         base += nw * 32) {
        const uint64_t i = base + lane;
        uint64_t q = ~0ull;
        if (i < R.count) {
            q = R.order ? (uint64_t)R.order[R.begin + i] : R.begin + i;
            if (q >= P.n) q = ~0ull;   /* orders are checked on the host; never index outside */
        }
        uint32_t tid = 0, live = 0, w0 = 0, p0 = 0, np = 0, T = 0;
        uint32_t t0 = 0, t1 = 0, t2 = 0;
        if (q != ~0ull) {
            tid = P.task[q];
            live = P.live[q];
            w0 = P.rdl[q];
            if (task.active[tid] && w0) {
                const uint32_t m = (live >> 1) & 127u;
                p0 = c_pr_off_g[m * 8 + w0];
                np = c_pr_off_g[m * 8 + w0 + 1] - p0;
                nev += __ldg(c_ev_sd1 + m * 8 + w0);
                T = (uint32_t)task.T[tid];
                t0 = task.target[tid * 32];
                if (FT >= 2) t1 = task.target[tid * 32 + 1];
                if (FT >= 3) t2 = task.target[tid * 32 + 2];
            }
        }
        __syncwarp();
        if (np) {
            /* the prefix's probe: registers 2h and 2h+1 on tests 0..3 in
               16-byte piece h */
            const uint4 *pp = reinterpret_cast<const uint4 *>(P.probe + q * 32);
#pragma unroll
            for (int h = 0; h < 4; h++) {
                const uint4 w = pp[h];
                const uint32_t lo[2] = {w.x, w.z}, hi[2] = {w.y, w.w};
#pragma unroll
                for (int k = 0; k < 2; k++) {
                    const int r = 2 * h + k;
                    if (r == 0) continue;
                    V[0][r][lane] = lo[k] & 0xFFFFu;
                    if (FT >= 2) V[FT >= 2 ? 1 : 0][r][lane] = lo[k] >> 16;
                    if (FT >= 3) V[FT >= 3 ? 2 : 0][r][lane] = hi[k] & 0xFFFFu;
                }
            }
        }
        __syncwarp();
        uint32_t jn = np;
#pragma unroll
        for (int o = 16; o; o >>= 1) jn = max(jn, __shfl_xor_sync(0xFFFFFFFFu, jn, o));
        for (uint32_t j = 0; j < jn; j++) {
            uint32_t hits = 0;
            if (j < np) {
                const uint32_t d = c_pr[p0 + j];
                const uint32_t a = d & 7u, b = (d >> 3) & 7u;
                const uint32_t e = (uint32_t)(uint16_t)(int16_t)(int8_t)(uint8_t)(d >> 16);
                hits = pair_hits(V[0][a][lane], V[0][b][lane], e, t0) & (d >> 6) & 0x3FFu;
                if (FT >= 2 && T >= 2 && hits)
                    hits &= pair_hits(V[FT >= 2 ? 1 : 0][a][lane], V[FT >= 2 ? 1 : 0][b][lane], e, t1);
                if (FT >= 3 && T >= 3 && hits)
                    hits &= pair_hits(V[FT >= 3 ? 2 : 0][a][lane], V[FT >= 3 ? 2 : 0][b][lane], e, t2);
            }
            uint32_t bal = __ballot_sync(0xFFFFFFFFu, hits != 0);
            while (bal) {
                const int L = __ffs(bal) - 1;
                bal &= bal - 1;
                uint32_t hj = __shfl_sync(0xFFFFFFFFu, hits, L);
                const unsigned long long qL = __shfl_sync(0xFFFFFFFFu, (unsigned long long)q, L);
                const uint32_t tidL = __shfl_sync(0xFFFFFFFFu, tid, L);
                const uint32_t liveL = __shfl_sync(0xFFFFFFFFu, live, L);
                const uint32_t pj = __shfl_sync(0xFFFFFFFFu, p0, L) + j;
                const uint32_t d = c_pr[pj];
                const uint32_t a = d & 7u, b = (d >> 3) & 7u;
                const uint32_t e = (uint32_t)(uint16_t)(int16_t)(int8_t)(uint8_t)(d >> 16);
                const int TL = task.T[tidL];
                const uint32_t tgt = lane < TL ? task.target[tidL * 32 + lane] : 0u;
                uint32_t x = 0, y = 0;
                if (!lean.up_regs) {
                    if (lane < TL) {
                        x = P.regs[(qL * 8 + a) * TPC + lane];
                        y = P.regs[(qL * 8 + b) * TPC + lane];
                    }
                } else {
                    /* a lean level: the prefix's registers are its parent's
                       but for the one its last instruction wrote */
                    const uint64_t pL = P.parent[qL];
                    const uint32_t uL = c_cand_uop[c_cand_off[(lean.up_live[pL] >> 1) & 127u] +
                                                   lean.cidx[qL]];
                    const uint32_t rdL = UOP_RD(uL);
                    if (lane < TL) {
                        const uint16_t *up = lean.up_regs + pL * 8 * TPC + lane;
                        const uint32_t w = pca_alu(UOP_OP(uL), up[UOP_A(uL) * TPC],
                                                   up[UOP_B(uL) * TPC], UOP_IMM(uL)) & 0xFFFFu;
                        x = a == rdL ? w : up[a * TPC];
                        y = b == rdL ? w : up[b * TPC];
                    }
                }
                const uint32_t vbase = c_vc_off[(liveL >> 1) & 127u];
                while (hj) {
                    const uint32_t k = (uint32_t)(__ffs(hj) - 1);
                    hj &= hj - 1;
                    bool ok = true;
                    if (lane < TL)
                        ok = (k == 9 ? ((x + e) & 0xFFFFu) : pca_alu(pair_op(k), x, y, 0)) == tgt;
                    if (__all_sync(0xFFFFFFFFu, ok) && lane == 0) {
                        const uint32_t cj = c_pr_cls[(uint64_t)pj * 10 + k];
                        record_solution(S, qL, 0, 0, cj, c_vc_first[vbase + cj]);
                    }
                }
            }
        }
    }
    /* the stage's evaluation count (k_count_evals' sum for these prefixes) */
    flush_evals(S, nev, lane);
}

/* The value of register x on test t after the middles (first FT tests):
   the innermost middle's own value, else the first middle's (suffix depth
   3), else the prefix's. */
template <int FT>
__device__ __forceinline__ uint32_t mid_val(const uint32_t (&V)[FT][8], int t, uint32_t x,
                                            uint32_t rdA, uint32_t vA, uint32_t rdB, uint32_t vB)
{
    return x == rdB ? vB : x == rdA ? vA : V[t][x];
}

/* Suffix depths 2 and 3 with a lane per instruction of the innermost
 * middle. SD = 2: a work item is a prefix and 32 of its middle candidates,
 * one per lane; SD = 3: a work item is a prefix and one first middle, whose
 * second middles the lanes take 32 at a time. A lane computes its middle's
 * value on the first FT tests from the prefix's probe (and the first
 * middle's, computed by every lane), applies k_suffix's rules (same-state
 * middles skipped under OEP; a write overwritten unread skips the branch;
 * the last instruction reads the innermost write and the one write still
 * owed a read, at most one), and walks the operand pairs of its mask that
 * read its middle's write, every op of a pair evaluated at once. A pair that
 * passes the first FT tests is checked on every test by the warp (lane =
 * test, the whole chain recomputed from the level's columns) and recorded
 * as k_suffix records it, so the records are the same. */
template <int TPC, int SD, int FT>
__global__ void __launch_bounds__(kThreads, 4)
k_suffix_mid_lanes(LevelDev P, TaskDev task, SolBuf S, uint32_t chunks_per_prefix, PrefixRange R)
{
    static_assert(SD == 2 || SD == 3, "middle lanes serve suffix depths 2 and 3");
    __shared__ uint32_t sV[kWarpsPerBlock][FT][8];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    uint32_t (&V)[FT][8] = sV[wib];
    const uint64_t nw = (uint64_t)gridDim.x * kWarpsPerBlock;
    const uint64_t items = R.count * chunks_per_prefix;
    uint64_t loaded = ~0ull;
    uint32_t cur_task = ~0u, T = 0, t0 = 0, t1 = 0, t2 = 0;
    bool cur_active = false;
    unsigned long long nev = 0;
    for (uint64_t it = (uint64_t)blockIdx.x * kWarpsPerBlock + wib; it < items; it += nw) {
        const uint64_t qi = it / chunks_per_prefix;
        const uint32_t ck = (uint32_t)(it - qi * chunks_per_prefix);
        const uint64_t q = R.order ? (uint64_t)R.order[R.begin + qi] : R.begin + qi;
        if (q >= P.n) continue;  /* orders are checked on the host; never index outside */
        const uint32_t tid = P.task[q];
        if (tid != cur_task) {
            cur_task = tid;
            cur_active = task.active[tid] != 0;
            T = (uint32_t)task.T[tid];
            t0 = task.target[tid * 32];
            if (FT >= 2) t1 = task.target[tid * 32 + 1];
            if (FT >= 3) t2 = task.target[tid * 32 + 2];
        }
        if (!cur_active) continue;
        const uint32_t live = P.live[q], w0 = P.rdl[q];
        const uint32_t m0 = (live >> 1) & 127u;
        const uint32_t cb0 = c_cand_off[m0], nc0 = c_cand_off[m0 + 1] - cb0;
        if (q != loaded) {
            __syncwarp();
            if (lane < FT * 8) V[lane >> 3][lane & 7] = P.probe[q * 32 + (lane & 7) * 4 + (lane >> 3)];
            __syncwarp();
            loaded = q;
        }
        /* the first middle: each lane's own (SD 2) or the work item's (SD 3) */
        const uint32_t i1 = SD == 2 ? ck * 32 + (uint32_t)lane : ck;
        if (SD == 3 && i1 >= nc0) continue;
        bool act1 = i1 < nc0;
        const uint32_t u1 = act1 ? c_cand_uop[cb0 + i1] : 0u;
        if (task.dedup_mid && (u1 >> 31)) act1 = false;
        const uint32_t rd1 = UOP_RD(u1);
        const uint32_t owe0 = w0 && !uop_reads(u1, w0) ? w0 : 0u;
        if (owe0 && rd1 == owe0) act1 = false;
        if (SD == 3 && !act1) continue;    /* uniform for the warp at SD 3 */
        uint32_t v1[FT];
#pragma unroll
        for (int t = 0; t < FT; t++)
            v1[t] = pca_alu(UOP_OP(u1), V[t][UOP_A(u1)], V[t][UOP_B(u1)], UOP_IMM(u1));
        /* (an inactive lane's micro-op is 0: rd 0, no bit to set) */
        const uint32_t m1 = rd1 ? (m0 | (1u << (rd1 - 1))) & 127u : m0;
        const uint32_t nc1 = SD == 3 ? c_cand_off[m1 + 1] - c_cand_off[m1] : 32u;
        for (uint32_t b2 = 0; b2 < nc1; b2 += 32) {
            /* the innermost middle of this lane and the last position's
               requirements */
            bool act = act1;
            uint32_t i2 = 0, u2 = 0, rdA = 8, rdB = rd1, need1 = rd1, need2 = owe0, m = m1;
            uint32_t vA[FT], vB[FT];
#pragma unroll
            for (int t = 0; t < FT; t++) {
                vA[t] = 0;
                vB[t] = v1[t];
            }
            if (SD == 3) {
                i2 = b2 + (uint32_t)lane;
                act = i2 < nc1;
                u2 = act ? c_cand_uop[c_cand_off[m1] + i2] : 0u;
                if (task.dedup_mid && (u2 >> 31)) act = false;
                const uint32_t rd2 = UOP_RD(u2);
                const uint32_t owe1 = uop_reads(u2, rd1) ? 0u : rd1;
                const uint32_t owe0b = owe0 && !uop_reads(u2, owe0) ? owe0 : 0u;
                if ((owe1 && rd2 == owe1) || (owe0b && rd2 == owe0b)) act = false;
                if (owe1 && owe0b) act = false;   /* three registers to read */
                need2 = owe1 ? owe1 : owe0b;
                need1 = rd2;
                m = rd2 ? (m1 | (1u << (rd2 - 1))) & 127u : m1;
                rdA = rd1;
                rdB = rd2;
#pragma unroll
                for (int t = 0; t < FT; t++) {
                    vA[t] = v1[t];
                    vB[t] = pca_alu(UOP_OP(u2), mid_val<FT>(V, t, UOP_A(u2), 8, 0, rd1, v1[t]),
                                    mid_val<FT>(V, t, UOP_B(u2), 8, 0, rd1, v1[t]), UOP_IMM(u2));
                }
            }
            uint32_t p0 = 0, np = 0;
            if (act) {
                p0 = c_pr_off_g[m * 8 + need1];
                np = c_pr_off_g[m * 8 + need1 + 1] - p0;
                if (!need2) nev += c_ev_sd1[m * 8 + need1];
            }
            uint32_t jn = np;
#pragma unroll
            for (int o = 16; o; o >>= 1) jn = max(jn, __shfl_xor_sync(0xFFFFFFFFu, jn, o));
            for (uint32_t j = 0; j < jn; j++) {
                uint32_t hits = 0;
                if (j < np) {
                    const uint32_t d = c_pr[p0 + j];
                    const uint32_t a = d & 7u, b = (d >> 3) & 7u;
                    if (!need2 || a == need2 || b == need2) {
                        if (need2) nev += __popc((d >> 6) & 0x3FFu);
                        const uint32_t e = (uint32_t)(uint16_t)(int16_t)(int8_t)(uint8_t)(d >> 16);
                        hits = pair_hits(mid_val<FT>(V, 0, a, rdA, vA[0], rdB, vB[0]),
                                         mid_val<FT>(V, 0, b, rdA, vA[0], rdB, vB[0]), e, t0) &
                               (d >> 6) & 0x3FFu;
                        if (FT >= 2 && T >= 2 && hits)
                            hits &= pair_hits(
                                mid_val<FT>(V, FT >= 2 ? 1 : 0, a, rdA, vA[FT >= 2 ? 1 : 0], rdB,
                                            vB[FT >= 2 ? 1 : 0]),
                                mid_val<FT>(V, FT >= 2 ? 1 : 0, b, rdA, vA[FT >= 2 ? 1 : 0], rdB,
                                            vB[FT >= 2 ? 1 : 0]), e, t1);
                        if (FT >= 3 && T >= 3 && hits)
                            hits &= pair_hits(
                                mid_val<FT>(V, FT >= 3 ? 2 : 0, a, rdA, vA[FT >= 3 ? 2 : 0], rdB,
                                            vB[FT >= 3 ? 2 : 0]),
                                mid_val<FT>(V, FT >= 3 ? 2 : 0, b, rdA, vA[FT >= 3 ? 2 : 0], rdB,
                                            vB[FT >= 3 ? 2 : 0]), e, t2);
                    }
                }
                uint32_t bal = __ballot_sync(0xFFFFFFFFu, hits != 0);
                while (bal) {
                    const int L = __ffs(bal) - 1;
                    bal &= bal - 1;
                    uint32_t hj = __shfl_sync(0xFFFFFFFFu, hits, L);
                    const uint32_t uL1 = __shfl_sync(0xFFFFFFFFu, u1, L);
                    const uint32_t uL2 = __shfl_sync(0xFFFFFFFFu, u2, L);
                    const uint32_t iL1 = __shfl_sync(0xFFFFFFFFu, i1, L);
                    const uint32_t iL2 = __shfl_sync(0xFFFFFFFFu, i2, L);
                    const uint32_t mL = __shfl_sync(0xFFFFFFFFu, m, L);
                    const uint32_t pj = __shfl_sync(0xFFFFFFFFu, p0, L) + j;
                    const uint32_t d = c_pr[pj];
                    const uint32_t a = d & 7u, b = (d >> 3) & 7u;
                    const uint32_t e = (uint32_t)(uint16_t)(int16_t)(int8_t)(uint8_t)(d >> 16);
                    /* the chain on test `lane`, from the level's columns */
                    uint32_t x = 0, y = 0, tg = 0;
                    if (lane < (int)T) {
                        const uint16_t *col = P.regs + q * 8 * TPC + lane;
                        const uint32_t r1 = UOP_RD(uL1);
                        const uint32_t m1v = pca_alu(UOP_OP(uL1), col[UOP_A(uL1) * TPC],
                                                     col[UOP_B(uL1) * TPC], UOP_IMM(uL1));
                        uint32_t r2 = 8, m2v = 0;
                        if (SD == 3) {
                            r2 = UOP_RD(uL2);
                            const uint32_t xa = UOP_A(uL2) == r1 ? m1v : col[UOP_A(uL2) * TPC];
                            const uint32_t xb = UOP_B(uL2) == r1 ? m1v : col[UOP_B(uL2) * TPC];
                            m2v = pca_alu(UOP_OP(uL2), xa, xb, UOP_IMM(uL2));
                        }
                        x = a == r2 ? m2v : a == r1 ? m1v : col[a * TPC];
                        y = b == r2 ? m2v : b == r1 ? m1v : col[b * TPC];
                        tg = task.target[tid * 32 + lane];
                    }
                    const uint32_t vbase = c_vc_off[mL];
                    while (hj) {
                        const uint32_t k = (uint32_t)(__ffs(hj) - 1);
                        hj &= hj - 1;
                        bool ok = true;
                        if (lane < (int)T)
                            ok = (k == 9 ? ((x + e) & 0xFFFFu) : pca_alu(pair_op(k), x, y, 0)) == tg;
                        if (__all_sync(0xFFFFFFFFu, ok) && lane == 0) {
                            const uint32_t cj = c_pr_cls[(uint64_t)pj * 10 + k];
                            record_solution(S, q, iL1, SD == 3 ? iL2 : 0u, cj, c_vc_first[vbase + cj]);
                        }
                    }
                }
            }
        }
    }
    flush_evals(S, nev, lane);
}

/* Value-class evaluations k_suffix<TPC, 1> runs over range R: a prefix of
   mask m whose last write is w0 scans the pair list of (m, w0), a root
   every class of its mask (c_ev_sd1, in global memory: the lanes read
   different entries). Added to S.evals, one atomic per warp. */
__global__ void k_count_evals(LevelDev P, TaskDev task, PrefixRange R, SolBuf S)
{
    const int lane = threadIdx.x & 31;
    unsigned long long nev = 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t n_round = (R.count + 31) & ~31ull;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_round; i += stride) {
        if (i >= R.count) continue;
        const uint64_t q = R.order ? (uint64_t)R.order[R.begin + i] : R.begin + i;
        if (q >= P.n || !task.active[P.task[q]]) continue;
        const uint32_t m = (P.live[q] >> 1) & 127u, w0 = P.rdl[q];
        nev += __ldg(c_ev_sd1 + m * 8 + w0);
    }
    flush_evals(S, nev, lane);
}

/* ---- recording: the reference's keys and records of level states --------- */

/* Engine column of each original test (the engine reorders tests). */
struct TestPos {
    uint8_t pos[MAX_TESTS];
};

/* FNV-1a-64 over the state's bytes in the reference's order (per original
 * test: r0..r7 low byte then high byte, then the flags): the oep hash; the
 * key adds live and depth (src/search_state.c:191-219). One thread per
 * state. */
template <int TPC>
__global__ void k_record_keys(LevelDev L, TestPos tp, int T, int depth, uint64_t *key,
                              uint64_t *oep)
{
    const uint64_t prime = 0x00000100000001B3ull;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < L.n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t h = 0xCBF29CE484222325ull;
        for (int u = 0; u < T; u++) {
            const int c = tp.pos[u];
#pragma unroll
            for (int r = 0; r < 8; r++) {
                const uint32_t v = L.regs[(i * 8 + r) * TPC + c];
                h = (h ^ (v & 0xFFu)) * prime;
                h = (h ^ (v >> 8)) * prime;
            }
            h = (h ^ L.flags[i * TPC + c]) * prime;
        }
        oep[i] = h;
        h = (h ^ L.live[i]) * prime;
        h = (h ^ (uint32_t)depth) * prime;
        key[i] = h;
    }
}

/* What the recording pass writes for one state (src/search_state.c:243-268). */
struct RecordMeta {
    uint32_t index;          /* state in its level */
    uint16_t parent_action;  /* 0xFFFF for the root */
    uint8_t  positive;
    int8_t   remaining;
};

/* One warp per record, lane = original test; `out` is zeroed beforehand. */
template <int TPC>
__global__ void k_record_states(LevelDev L, TestPos tp, int T, int depth, uint32_t task_id,
                                int target_depth, const RecordMeta *meta, uint64_t count,
                                const uint64_t *key, const uint64_t *oep,
                                dataset_state_record_t *out)
{
    const int lane = threadIdx.x & 31;
    const uint64_t nw = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < count; w += nw) {
        const RecordMeta m = meta[w];
        const uint64_t i = m.index;
        dataset_state_record_t &o = out[w];
        if (lane == 0) {
            o.state_hash = key[i];
            o.oep_hash = oep[i];
            o.task_id = task_id;
            o.parent_action = m.parent_action;
            o.depth = (uint8_t)depth;
            o.budget_left = (uint8_t)(target_depth - depth);
            o.live = L.live[i];
            o.can_finish_optimally = m.positive;
            o.remaining_steps = m.remaining;
        }
        if (lane < T) {
            const int c = tp.pos[lane];
#pragma unroll
            for (int r = 0; r < 8; r++) o.regs[lane][r] = L.regs[(i * 8 + r) * TPC + c];
            o.flags[lane] = L.flags[i * TPC + c];
        }
    }
}

}  // namespace pcagb
