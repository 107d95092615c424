/*
 * branch.cu -- the reference solver's branch mode on the GPU: kernels with
 * CMP and forward BR (and DIV/MOD), searched by iterative deepening with the
 * reference's candidate rules and its observational-equivalence pruning
 * (tools/enumerate.c:204-260 candidates, :405-455 search, :54-77 pruner,
 * :262-286 output check; src/vm.c:59-203 semantics).
 *
 * A straight-line state is not enough once a forward branch is taken: the
 * instructions it jumps over are not executed. Each test therefore carries,
 * besides r0..r7 and the flags, the kernel position where it resumes
 * (`skip`): an instruction at position p runs for test t only if
 * skip[t] <= p; a taken BR at p sets skip[t] = p + 1 + offset; a division
 * by zero stops the test for good (skip = 255; the VM faults and the test
 * can no longer pass). Forward offsets never reach past the OUT at the end
 * of a complete program, so every test that did not fault executes OUT.
 *
 * Pruning follows the reference: the key of a child is its registers and
 * flags on every test (the reference hashes the VM state after running the
 * partial program; the pending-jump state is not part of it), BR children
 * are never pruned and never enter the table, and among equal keys the
 * first child in depth-first order is kept. Here the key is exact (64-bit
 * hash plus a full compare on every tag match) where the reference keeps 32
 * bits. The candidate list of a position depends on the depth being
 * searched (BR offsets reach at most to the end of the kernel), so every
 * depth of the iterative deepening builds its levels afresh.
 *
 * Levels live in stream-ordered device allocations on the engine's stream;
 * every launch goes to that stream.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/pca_gb300.h"
#include "pca_isa.h"
#include "scan.cuh"

namespace {

constexpr int kOpDiv = 0x05, kOpMod = 0x06, kOpCmp = 0x0D, kOpBr = 0x13;
constexpr uint8_t kFault = 255;
constexpr int kWarps = 8;
constexpr int kBThreads = 32 * kWarps;
/* Last-position children above which the last level is not built (its
   table alone would take 16 bytes per child). */
constexpr uint64_t kMaterializeMax = 1ull << 26;

std::string g_berr;
void set_berr(const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_berr = buf;
}

#define BCK(call)                                                                         \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) {                                                          \
            set_berr("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__,   \
                     __LINE__);                                                           \
            return PCAGB_ECUDA;                                                           \
        }                                                                                 \
    } while (0)

/* ---- candidates (tools/enumerate.c:204-260), per liveness mask ---------- */

/* For each of the 128 masks of live r1..r7: the ALU and CMP candidates
   (before the BR block) and the LDI and ADDI candidates (after it). The BR
   block of a position with `mf` forward offsets is cond 1..6 x offset
   1..mf, in that order. */
struct BranchTables {
    std::vector<uint32_t> pre_off, post_off;  /* size 129 */
    std::vector<uint16_t> pre, post;
};

const BranchTables &branch_tables()
{
    static BranchTables *t = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        t = new BranchTables();
        static const uint8_t alu[] = {PCA_OP_ADD, PCA_OP_SUB, PCA_OP_MUL, kOpDiv, kOpMod,
                                      PCA_OP_AND, PCA_OP_OR, PCA_OP_XOR, PCA_OP_SHL,
                                      PCA_OP_SHR, PCA_OP_ASR};
        static const int commut[] = {1, 0, 1, 0, 0, 1, 1, 1, 0, 0, 0};
        static const uint8_t ldi[] = {0, 1, 2, 3, 4, 5, 8, 16, 32, 64, 128, 255};
        static const int8_t addi[] = {-1, 1, -2, 2, -3, 3};
        t->pre_off.assign(129, 0);
        t->post_off.assign(129, 0);
        for (int m = 0; m < 128; m++) {
            const unsigned live = (unsigned)m << 1;
            t->pre_off[m] = (uint32_t)t->pre.size();
            for (int oi = 0; oi < 11; oi++) {
                const int op = alu[oi];
                for (int rd = 1; rd < 8; rd++)
                    for (int rs = 0; rs < 8; rs++) {
                        if (rs && !(live >> rs & 1u)) continue;
                        for (int rt = commut[oi] ? rs : 0; rt < 8; rt++) {
                            if (rt && !(live >> rt & 1u)) continue;
                            if (rs == 0 && rt == 0) continue;
                            if (op == PCA_OP_ADD && rs == rd && rt == 0) continue;
                            if (op == PCA_OP_ADD && rt == rd && rs == 0) continue;
                            if (op == PCA_OP_SUB && rs == rd && rt == 0) continue;
                            if (op == PCA_OP_MUL && (rs == 0 || rt == 0)) continue;
                            if ((op == kOpDiv || op == kOpMod) && rt == 0) continue;
                            if ((op == PCA_OP_SHL || op == PCA_OP_SHR || op == PCA_OP_ASR) && rt == 0)
                                continue;
                            t->pre.push_back((uint16_t)PCA_ENC_R(op, rd, rs, rt));
                        }
                    }
            }
            for (int rd = 0; rd < 8; rd++) {
                if (rd && !(live >> rd & 1u)) continue;
                for (int rs = 0; rs < 8; rs++) {
                    if (rs && !(live >> rs & 1u)) continue;
                    if (rd == 0 && rs == 0) continue;
                    if (rd == rs) continue;
                    t->pre.push_back((uint16_t)PCA_ENC_R(kOpCmp, rd, rs, 0));
                }
            }
            t->post_off[m] = (uint32_t)t->post.size();
            for (int rd = 1; rd < 8; rd++)
                for (uint8_t v : ldi) t->post.push_back((uint16_t)PCA_ENC_I(PCA_OP_LDI, rd, v));
            for (int rd = 1; rd < 8; rd++) {
                if (!(live >> rd & 1u)) continue;
                for (int8_t v : addi)
                    t->post.push_back((uint16_t)PCA_ENC_I(PCA_OP_ADDI, rd, (uint8_t)v));
            }
        }
        t->pre_off[128] = (uint32_t)t->pre.size();
        t->post_off[128] = (uint32_t)t->post.size();
    });
    return *t;
}

struct BTab {
    const uint32_t *pre_off, *post_off;
    const uint16_t *pre, *post;
    int mf;  /* forward offsets at this position */
};

__host__ __device__ __forceinline__ uint32_t bcount(const BTab &b, uint32_t m)
{
    return (b.pre_off[m + 1] - b.pre_off[m]) + 6u * (uint32_t)b.mf + (b.post_off[m + 1] - b.post_off[m]);
}

__host__ __device__ __forceinline__ uint16_t bcand(const BTab &b, uint32_t m, uint32_t c)
{
    const uint32_t npre = b.pre_off[m + 1] - b.pre_off[m];
    if (c < npre) return b.pre[b.pre_off[m] + c];
    c -= npre;
    const uint32_t nbr = 6u * (uint32_t)b.mf;
    if (c < nbr) {
        const uint32_t cond = 1 + c / (uint32_t)b.mf, off = 1 + c % (uint32_t)b.mf;
        return (uint16_t)PCA_ENC_I(kOpBr, cond, off);
    }
    return b.post[b.post_off[m] + (c - nbr)];
}

/* ---- one instruction on one test (src/vm.c:59-203) ----------------------- */

__device__ __forceinline__ uint32_t zn(uint32_t v)
{
    return (v == 0 ? PCA_FZ : 0u) | (v & 0x8000u ? PCA_FN : 0u);
}

__device__ __forceinline__ uint32_t f_add(uint32_t a, uint32_t b)
{
    const uint32_t full = a + b, r = full & 0xFFFFu;
    return zn(r) | (full > 0xFFFFu ? PCA_FC : 0u) | ((~(a ^ b) & (a ^ r) & 0x8000u) ? PCA_FV : 0u);
}

__device__ __forceinline__ uint32_t f_sub(uint32_t a, uint32_t b)
{
    const uint32_t r = (a - b) & 0xFFFFu;
    return zn(r) | (a >= b ? PCA_FC : 0u) | (((a ^ b) & (a ^ r) & 0x8000u) ? PCA_FV : 0u);
}

/* Apply insn at kernel position p: writes the changed register value to
   *val (or leaves it), the flags to *f and the resume position to *skip.
   Returns the register written (0 = none). */
__device__ __forceinline__ uint32_t bexec(uint32_t insn, uint32_t p, const uint32_t *R, uint32_t f0,
                                          uint32_t skip0, uint32_t *val, uint32_t *f, uint32_t *skip)
{
    *f = f0;
    *skip = skip0;
    if (skip0 > p) return 0;  /* jumped over, or stopped by a fault */
    const uint32_t op = insn >> 11, rd = (insn >> 8) & 7u, rs = (insn >> 5) & 7u, rt = (insn >> 2) & 7u;
    const uint32_t imm = insn & 0xFFu;
    const uint32_t a = R[rs], b = R[rt];
    uint32_t v = 0;
    switch (op) {
    case PCA_OP_ADD: v = (a + b) & 0xFFFFu; *f = f_add(a, b); break;
    case PCA_OP_SUB: v = (a - b) & 0xFFFFu; *f = f_sub(a, b); break;
    case PCA_OP_MUL: {
        const uint32_t prod = a * b;
        v = prod & 0xFFFFu;
        *f = zn(v) | (prod > 0xFFFFu ? PCA_FC : 0u);
        break;
    }
    case kOpDiv:
    case kOpMod:
        if (b == 0) {
            *skip = kFault;
            return 0;
        }
        {
            const int sa = (int)(int16_t)(uint16_t)a, sb = (int)(int16_t)(uint16_t)b;
            v = (uint32_t)(uint16_t)(op == kOpDiv ? sa / sb : sa % sb);
        }
        *f = zn(v);
        break;
    case PCA_OP_AND: v = a & b; *f = zn(v); break;
    case PCA_OP_OR:  v = a | b; *f = zn(v); break;
    case PCA_OP_XOR: v = a ^ b; *f = zn(v); break;
    case PCA_OP_SHL: v = (a << (b & 15u)) & 0xFFFFu; *f = zn(v); break;
    case PCA_OP_SHR: v = a >> (b & 15u); *f = zn(v); break;
    case PCA_OP_ASR: v = (uint32_t)(uint16_t)((int16_t)(uint16_t)a >> (b & 15u)); *f = zn(v); break;
    case kOpCmp: *f = f_sub(R[rd], a); return 0;
    case kOpBr: {
        const uint32_t Z = f0 & PCA_FZ, N = (f0 & PCA_FN) != 0, C = f0 & PCA_FC,
                       V = (f0 & PCA_FV) != 0;
        bool take = false;
        switch (rd) {
        case 0: take = true; break;
        case 1: take = Z != 0; break;
        case 2: take = Z == 0; break;
        case 3: take = N != V; break;
        case 4: take = N == V; break;
        case 5: take = C == 0; break;
        case 6: take = C != 0; break;
        }
        if (take) *skip = p + 1 + (uint32_t)(int32_t)(int8_t)(uint8_t)imm;
        return 0;
    }
    case PCA_OP_LDI: v = imm; break;
    case PCA_OP_ADDI: {
        const uint32_t s = (uint32_t)(int32_t)(int8_t)(uint8_t)imm & 0xFFFFu;
        *f = f_add(R[rd], s);
        v = (R[rd] + s) & 0xFFFFu;
        break;
    }
    default: return 0;
    }
    *val = v;
    return rd;
}

/* ---- levels ---------------------------------------------------------------- */

struct BLevel {
    uint64_t n = 0;
    uint16_t *regs = nullptr;   /* [n][8][TP] */
    uint8_t *flags = nullptr;   /* [n][TP] */
    uint8_t *skip = nullptr;    /* [n][TP] */
    uint8_t *live = nullptr;    /* [n] */
    uint32_t *parent = nullptr;
    uint16_t *cidx = nullptr;
    uint64_t *child_off = nullptr; /* [n+1] */
    uint64_t children = 0;
};

struct BDev {
    const uint16_t *regs;
    const uint8_t *flags, *skip, *live;
    const uint64_t *child_off;
    uint64_t n;
};

__device__ __forceinline__ uint64_t bmix(uint64_t x)
{
    x ^= x >> 33;
    x *= 0xFF51AFD7ED558CCDull;
    x ^= x >> 33;
    x *= 0xC4CEB9FE1A85EC53ull;
    x ^= x >> 33;
    return x;
}

/* Key of a child: registers and flags of every test (not the resume
   position), hashed per test then mixed. */
template <int TP>
__device__ uint64_t child_key(const BDev &P, uint64_t q, uint32_t insn, uint32_t p, int T)
{
    uint64_t h = 0x9E3779B97F4A7C15ull;
    for (int t = 0; t < T; t++) {
        uint32_t R[8];
#pragma unroll
        for (int r = 0; r < 8; r++) R[r] = P.regs[(q * 8 + r) * TP + t];
        uint32_t v = 0, f, sk;
        const uint32_t rd = bexec(insn, p, R, P.flags[q * TP + t], P.skip[q * TP + t], &v, &f, &sk);
        if (rd) R[rd] = v;
        uint64_t x = (uint64_t)f << 48 | (uint64_t)t << 56;
        x ^= bmix((uint64_t)R[1] | (uint64_t)R[2] << 16 | (uint64_t)R[3] << 32 | (uint64_t)R[4] << 48);
        x ^= bmix(((uint64_t)R[5] | (uint64_t)R[6] << 16 | (uint64_t)R[7] << 32) + 0x51ull);
        h = bmix(h ^ x) + 0x2545F4914F6CDD1Dull;
    }
    return h;
}

/* Two children equal in registers and flags on every test (warp-wide: lane = test). */
template <int TP>
__device__ bool bchild_equal(const BDev &P, uint64_t qa, uint32_t ia, uint64_t qb, uint32_t ib,
                             uint32_t p, int T, int lane)
{
    bool ok = true;
    if (lane < T) {
        uint32_t A[8], B[8];
#pragma unroll
        for (int r = 0; r < 8; r++) {
            A[r] = P.regs[(qa * 8 + r) * TP + lane];
            B[r] = P.regs[(qb * 8 + r) * TP + lane];
        }
        uint32_t va = 0, fa, sa, vb = 0, fb, sb;
        const uint32_t ra = bexec(ia, p, A, P.flags[qa * TP + lane], P.skip[qa * TP + lane], &va, &fa, &sa);
        const uint32_t rb = bexec(ib, p, B, P.flags[qb * TP + lane], P.skip[qb * TP + lane], &vb, &fb, &sb);
        if (ra) A[ra] = va;
        if (rb) B[rb] = vb;
        ok = fa == fb;
#pragma unroll
        for (int r = 1; r < 8; r++) ok &= A[r] == B[r];
    }
    return __all_sync(0xFFFFFFFFu, ok);
}

__global__ void k_bchild_counts(BDev P, BTab tab, uint64_t *cnt)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < P.n;
         i += (uint64_t)gridDim.x * blockDim.x)
        cnt[i] = bcount(tab, (P.live[i] >> 1) & 127u);
}

constexpr uint64_t kBRefMask = (1ull << 40) - 1;
constexpr uint32_t kBMaxProbes = 1u << 16;

/* One warp per parent, one lane per candidate (32 at a time): BR children
   are kept (their bit set at once), the others go through the exact table. */
template <int TP>
__global__ void __launch_bounds__(kBThreads)
k_bexpand(BDev P, BTab tab, int T, uint32_t p, unsigned long long *table, uint64_t tmask,
          uint32_t *bitmap, uint32_t *status)
{
    const int lane = threadIdx.x & 31;
    const uint64_t nw = (uint64_t)gridDim.x * kWarps;
    for (uint64_t q = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < P.n; q += nw) {
        const uint32_t m = (P.live[q] >> 1) & 127u;
        const uint32_t nc = bcount(tab, m);
        for (uint32_t c0 = 0; c0 < nc; c0 += 32) {
            const uint32_t c = c0 + lane;
            const bool valid = c < nc;
            const uint32_t insn = valid ? bcand(tab, m, c) : 0u;
            const bool br = valid && (insn >> 11) == (uint32_t)kOpBr;
            if (br) {
                const uint64_t L = P.child_off[q] + c;
                atomicOr(&bitmap[L >> 5], 1u << (L & 31));
            }
            uint64_t H = 0;
            if (valid && !br) H = child_key<TP>(P, q, insn, p, T);
            const uint64_t ref = (q << 12) | c;
            const unsigned long long mine = ((H >> 40) << 40) | (ref + 1);
            uint64_t idx = H & tmask;
            uint32_t probes = 0;
            bool done = !valid || br;
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
                uint32_t req = __ballot_sync(0xFFFFFFFFu, needcmp);
                bool eq = false;
                while (req) {
                    const int j = __ffs(req) - 1;
                    req &= req - 1;
                    const uint32_t ij = __shfl_sync(0xFFFFFFFFu, insn, j);
                    const unsigned long long sj = __shfl_sync(0xFFFFFFFFu, s, j);
                    const uint64_t oref = (sj & kBRefMask) - 1;
                    const uint64_t qb = oref >> 12;
                    const uint32_t ib = bcand(tab, (P.live[qb] >> 1) & 127u, (uint32_t)(oref & 4095));
                    const bool e = bchild_equal<TP>(P, q, ij, qb, ib, p, T, lane);
                    if (lane == j) eq = e;
                }
                if (!done) {
                    if (needcmp && eq) {
                        uint64_t oref = (s & kBRefMask) - 1;
                        while (ref < oref) {
                            const unsigned long long old = atomicCAS(&table[idx], s, mine);
                            if (old == s) break;
                            s = old;
                            oref = (s & kBRefMask) - 1;
                        }
                        done = true;
                    } else {
                        idx = (idx + 1) & tmask;
                        if (++probes >= kBMaxProbes) {
                            atomicOr(status, 1u);
                            done = true;
                        }
                    }
                }
            }
        }
    }
}

__global__ void k_bmark(const unsigned long long *table, uint64_t slots, const uint64_t *child_off,
                        uint32_t *bitmap)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < slots;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned long long s = table[i];
        if (!s) continue;
        const uint64_t ref = (s & kBRefMask) - 1;
        const uint64_t L = child_off[ref >> 12] + (ref & 4095);
        atomicOr(&bitmap[L >> 5], 1u << (L & 31));
    }
}

__global__ void k_bpopc(const uint32_t *bitmap, uint64_t words, uint64_t *off)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < words;
         i += (uint64_t)gridDim.x * blockDim.x)
        off[i] = __popc(bitmap[i]);
}

/* One warp per parent: its kept children, lane = test. */
template <int TP>
__global__ void __launch_bounds__(kBThreads)
k_bmaterialize(BDev P, BTab tab, int T, uint32_t p, const uint32_t *bitmap,
               const uint64_t *word_rank, BLevel C)
{
    const int lane = threadIdx.x & 31;
    const uint64_t nw = (uint64_t)gridDim.x * kWarps;
    for (uint64_t q = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < P.n; q += nw) {
        const uint32_t m = (P.live[q] >> 1) & 127u;
        const uint32_t nc = bcount(tab, m);
        const uint64_t base = P.child_off[q];
        uint32_t R[8] = {0, 0, 0, 0, 0, 0, 0, 0}, f0 = 0, s0 = 0;
        if (lane < TP) {
#pragma unroll
            for (int r = 0; r < 8; r++) R[r] = P.regs[(q * 8 + r) * TP + lane];
            f0 = P.flags[q * TP + lane];
            s0 = P.skip[q * TP + lane];
        }
        for (uint32_t c = 0; c < nc; c++) {
            const uint64_t L = base + c;
            if (!(bitmap[L >> 5] >> (L & 31) & 1u)) continue;
            const uint64_t k = word_rank[L >> 5] + __popc(bitmap[L >> 5] & ((1u << (L & 31)) - 1u));
            const uint32_t insn = bcand(tab, m, c);
            uint32_t v = 0, f = f0, sk = s0, rd = 0;
            if (lane < T) rd = bexec(insn, p, R, f0, s0, &v, &f, &sk);
            if (lane < TP) {
#pragma unroll
                for (int r = 0; r < 8; r++)
                    C.regs[(k * 8 + r) * TP + lane] = (uint16_t)(lane < T ? (rd == (uint32_t)r ? v : R[r]) : 0u);
                C.flags[k * TP + lane] = (uint8_t)(lane < T ? f : 0u);
                C.skip[k * TP + lane] = (uint8_t)(lane < T ? sk : 0u);
            }
            if (lane == 0) {
                const uint32_t op = insn >> 11, rdi = (insn >> 8) & 7u;
                uint32_t nl = P.live[q];
                if (op != (uint32_t)kOpCmp && op != (uint32_t)kOpBr && rdi != 0) nl |= 1u << rdi;
                C.live[k] = (uint8_t)nl;
                C.parent[k] = (uint32_t)q;
                C.cidx[k] = (uint16_t)c;
            }
        }
    }
}

/* Output check of a complete kernel (tools/enumerate.c:262-286 with
   tasks/spec.c:187-212): OUT r passes on a test that did not fault and
   holds the target in r. Bit r of mask[i] is set when it passes on all. */
template <int TP>
__global__ void k_bleaf(BDev P, int T, const uint32_t *target, uint8_t *mask)
{
    const int lane = threadIdx.x & 31;
    const uint64_t nw = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t q = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < P.n; q += nw) {
        const uint32_t live = P.live[q];
        uint32_t ok = 0;
        for (int r = 1; r < 8; r++) {
            if (!(live >> r & 1u)) continue;
            bool good = true;
            if (lane < T)
                good = P.skip[q * TP + lane] != kFault && P.regs[(q * 8 + r) * TP + lane] == target[lane];
            if (__all_sync(0xFFFFFFFFu, good)) ok |= 1u << r;
        }
        if (lane == 0) mask[q] = (uint8_t)ok;
    }
}

/* ---- the last position without its level ------------------------------------ */

/* A child of the last position whose registers hold the target on every
   test (live or not, faulted or not): its linear child index (depth-first
   order), key, parent, candidate, and the registers it solves for (0 when
   it faulted or the matching registers are not live: it cannot solve, but
   it may be the depth-first first of a solving child's key). */
struct BSol {
    uint64_t L;
    uint64_t key;
    uint32_t q;
    uint16_t c;
    uint8_t mask;
    uint8_t pad;
};

/* One warp per parent, one lane per last-position candidate: the output
   check of every complete kernel without materializing the last level. A
   register other than the written one holds the target when the parent's
   column already does on every test; the written one when its new column
   does; a test that faults (here or before) fails every register. Every
   child whose registers hold the target is recorded, solving or not: a
   child with the same state as a solving one holds the same registers, so
   the records contain the depth-first first child of every solving state
   (the one the pruner keeps) without a pass over all children. */
template <int TP>
__global__ void __launch_bounds__(kBThreads)
k_bsuffix(BDev P, BTab tab, int T, uint32_t p, const uint32_t *target, BSol *out,
          unsigned long long *count, uint64_t cap, uint64_t q_begin, uint64_t q_end)
{
    __shared__ uint32_t sRall[kWarps][8][TP + 1];
    __shared__ uint32_t sFall[kWarps][TP], sSall[kWarps][TP];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    uint32_t (&sR)[8][TP + 1] = sRall[wib];
    uint32_t *sF = sFall[wib], *sS = sSall[wib];
    const uint64_t nw = (uint64_t)gridDim.x * kWarps;
    const uint64_t qe = q_end < P.n ? q_end : P.n;
    for (uint64_t q = q_begin + (((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5); q < qe;
         q += nw) {
        uint32_t pm = 0;
        bool faulted = false;
        for (int r = 1; r < 8; r++) {
            bool good = true;
            if (lane < T) good = P.regs[(q * 8 + r) * TP + lane] == target[lane];
            if (__all_sync(0xFFFFFFFFu, good)) pm |= 1u << r;
        }
        if (lane < T) faulted = P.skip[q * TP + lane] == kFault;
        const bool pfault = __any_sync(0xFFFFFFFFu, faulted);
        /* the parent in shared memory: every lane reads test t of it */
        __syncwarp();
        if (lane < TP) {
#pragma unroll
            for (int r = 0; r < 8; r++) sR[r][lane] = P.regs[(q * 8 + r) * TP + lane];
            sF[lane] = P.flags[q * TP + lane];
            sS[lane] = P.skip[q * TP + lane];
        }
        __syncwarp();
        const uint32_t live = P.live[q];
        const uint32_t m = (live >> 1) & 127u;
        const uint32_t nc = bcount(tab, m);
        for (uint32_t c0 = 0; c0 < nc; c0 += 32) {
            const uint32_t c = c0 + lane;
            if (c >= nc) continue;
            const uint32_t insn = bcand(tab, m, c);
            const uint32_t op = insn >> 11, rdi = (insn >> 8) & 7u;
            const uint32_t wr = (op != (uint32_t)kOpCmp && op != (uint32_t)kOpBr && rdi != 0) ? rdi : 0u;
            /* a register the child leaves as the parent's can hold the
               target only where the parent's column does */
            const bool kept = (pm & ~(1u << wr) & 0xFEu) != 0;
            if (!kept && !wr) continue;
            bool match = wr != 0, fault = pfault;
            for (int t = 0; t < T; t++) {
                uint32_t R[8];
#pragma unroll
                for (int r = 0; r < 8; r++) R[r] = sR[r][t];
                uint32_t v = 0, f, sk;
                const uint32_t rd = bexec(insn, p, R, sF[t], sS[t], &v, &f, &sk);
                if (sk == kFault) fault = true;
                if (wr) match &= (rd == wr ? v : R[wr]) == target[t];
                /* nothing left to record once the written register missed
                   and no other register holds the target */
                if (!match && !kept) break;
            }
            uint32_t any = pm & ~(1u << wr);
            if (match) any |= 1u << wr;
            any &= 0xFEu;
            if (!any) continue;
            const uint32_t clive = live | (wr ? 1u << wr : 0u);
            const uint32_t mask = fault ? 0u : (any & clive);
            const unsigned long long i = atomicAdd(count, 1ull);
            if (i < cap) {
                BSol s;
                s.L = P.child_off[q] + c;
                s.key = child_key<TP>(P, q, insn, p, T);
                s.q = (uint32_t)q;
                s.c = (uint16_t)c;
                s.mask = (uint8_t)mask;
                s.pad = 0;
                out[i] = s;
            }
        }
    }
}

/* Pairs of last-position children (parent, candidate) compared in full,
   one warp per pair: eq[i] = 1 when equal in registers and flags. */
template <int TP>
__global__ void k_bpairs_equal(BDev P, BTab tab, int T, uint32_t p, const uint4 *pairs, uint64_t n,
                               uint8_t *eq)
{
    const int lane = threadIdx.x & 31;
    const uint64_t nw = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t i = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += nw) {
        const uint4 pr = pairs[i];
        const uint32_t ia = bcand(tab, (P.live[pr.x] >> 1) & 127u, pr.y);
        const uint32_t ib = bcand(tab, (P.live[pr.z] >> 1) & 127u, pr.w);
        const bool e = bchild_equal<TP>(P, pr.x, ia, pr.z, ib, p, T, lane);
        if (lane == 0) eq[i] = e ? 1 : 0;
    }
}

/* The tree links of solving children, gathered on the device so that no
   level's links cross the bus: for solution i (state qs[i] of level K-1 and
   candidate c), out[i][d] = (live mask of its level-d ancestor) << 16 |
   (candidate index that ancestor's child on the path took), d = 0..K-1. */
struct BPath {
    const uint32_t *parent[16];
    const uint16_t *cidx[16];
    const uint8_t *live[16];
};

__global__ void k_bpath(BPath L, int K, const uint32_t *qs, const uint16_t *cs, int ns,
                        uint32_t *out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
        uint64_t st = qs[i];
        out[(size_t)i * K + K - 1] = (uint32_t)L.live[K - 1][st] << 16 | cs[i];
        for (int d = K - 1; d >= 1; d--) {
            const uint32_t par = L.parent[d][st];
            out[(size_t)i * K + d - 1] = (uint32_t)L.live[d - 1][par] << 16 | L.cidx[d][st];
            st = par;
        }
    }
}

/* ---- host driver ----------------------------------------------------------- */

struct BranchRun {
    cudaStream_t st;
    int sms;
    int TP;
    int T;
    const task_spec_t *task;
    uint32_t *d_target = nullptr;
    uint32_t *d_pre_off = nullptr, *d_post_off = nullptr;
    uint16_t *d_pre = nullptr, *d_post = nullptr;
    uint32_t *d_status = nullptr;
    std::vector<void *> allocs;
    uint64_t h2d = 0, d2h = 0;
    int launches = 0;

    ~BranchRun()
    {
        release(0);
        cudaStreamSynchronize(st);
    }
    /* free the allocations made after the first `keep` */
    void release(size_t keep)
    {
        while (allocs.size() > keep) {
            cudaFreeAsync(allocs.back(), st);
            allocs.pop_back();
        }
    }
    template <class X>
    X *alloc(size_t count)
    {
        void *p = nullptr;
        if (cudaMallocAsync(&p, std::max<size_t>(count * sizeof(X), 16), st) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        allocs.push_back(p);
        return (X *)p;
    }
    BTab tab(int mf) const { return BTab{d_pre_off, d_post_off, d_pre, d_post, mf}; }
    int grid(int per_sm) const { return sms * per_sm; }
};

BDev bdev(const BLevel &L) { return BDev{L.regs, L.flags, L.skip, L.live, L.child_off, L.n}; }

int alloc_blevel(BranchRun &b, BLevel &L, uint64_t n)
{
    L.n = n;
    L.regs = b.alloc<uint16_t>(n * 8 * b.TP);
    L.flags = b.alloc<uint8_t>(n * b.TP);
    L.skip = b.alloc<uint8_t>(n * b.TP);
    L.live = b.alloc<uint8_t>(n);
    L.parent = b.alloc<uint32_t>(n);
    L.cidx = b.alloc<uint16_t>(n);
    if (!L.regs || !L.flags || !L.skip || !L.live || !L.parent || !L.cidx) {
        set_berr("device memory exhausted for a level of %llu states", (unsigned long long)n);
        return PCAGB_ENOMEM;
    }
    return PCAGB_OK;
}

int blaunch(BranchRun &b)
{
    b.launches++;
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) {
        set_berr("kernel launch failed: %s", cudaGetErrorString(err));
        return PCAGB_ECUDA;
    }
    return PCAGB_OK;
}

/* Exclusive scan of a[0..n) in place on the stream (nothing read back). */
int bscan(BranchRun &b, uint64_t *a, uint64_t n)
{
    if (n == 0) return PCAGB_OK;
    const uint64_t nb = (n + kScanBlock - 1) / kScanBlock;
    uint64_t *sums = b.alloc<uint64_t>(nb + 1);
    if (!sums) { set_berr("device memory exhausted in a scan"); return PCAGB_ENOMEM; }
    k_scan_local<<<(unsigned)nb, 256, 0, b.st>>>(a, n, sums);
    int rc = blaunch(b);
    if (rc) return rc;
    if (nb > 1) {
        rc = bscan(b, sums, nb);
        if (rc) return rc;
        k_scan_add<<<(unsigned)nb, 256, 0, b.st>>>(a, n, sums);
        rc = blaunch(b);
    }
    return rc;
}

/* Expand level P (position p of a depth-K pass) into C. Fills the number of
   generated children. */
/* Children of every state of P at a position with mf forward offsets:
   P.child_off (exclusive scan) and P.children. */
int count_bchildren(BranchRun &b, BLevel &P, int mf)
{
    const BTab tab = b.tab(mf);
    P.child_off = b.alloc<uint64_t>(P.n + 1);
    if (!P.child_off) { set_berr("device memory exhausted"); return PCAGB_ENOMEM; }
    BCK(cudaMemsetAsync(P.child_off + P.n, 0, 8, b.st));
    k_bchild_counts<<<b.grid(2), 256, 0, b.st>>>(bdev(P), tab, P.child_off);
    int rc = blaunch(b);
    if (rc) return rc;
    /* exclusive scan on the device; the total lands in child_off[n] */
    rc = bscan(b, P.child_off, P.n + 1);
    if (rc) return rc;
    uint64_t total = 0;
    BCK(cudaMemcpyAsync(&total, P.child_off + P.n, 8, cudaMemcpyDeviceToHost, b.st));
    BCK(cudaStreamSynchronize(b.st));
    b.d2h += 8;
    P.children = total;
    if (P.n >= (1ull << 28) || total >= (1ull << 38)) {
        set_berr("level too large (%llu states, %llu children)", (unsigned long long)P.n,
                 (unsigned long long)total);
        return PCAGB_ENOMEM;
    }
    return PCAGB_OK;
}

int build_blevel(BranchRun &b, BLevel &P, uint32_t p, int mf, BLevel &C)
{
    const BTab tab = b.tab(mf);
    int rc = P.child_off ? PCAGB_OK : count_bchildren(b, P, mf);
    if (rc) return rc;
    const uint64_t total = P.children;
    const uint64_t words = (total + 31) / 32;
    uint64_t slots = 1024;
    while (slots < 2 * total) slots <<= 1;
    uint32_t *bitmap = b.alloc<uint32_t>(words + 1);
    unsigned long long *table = b.alloc<unsigned long long>(slots);
    uint64_t *rank = b.alloc<uint64_t>(words + 1);
    if (!bitmap || !table || !rank) { set_berr("device memory exhausted expanding a level"); return PCAGB_ENOMEM; }
    BCK(cudaMemsetAsync(bitmap, 0, (words + 1) * 4, b.st));
    BCK(cudaMemsetAsync(table, 0, slots * 8, b.st));
    BCK(cudaMemsetAsync(b.d_status, 0, 4, b.st));
    if (b.TP == 16)
        k_bexpand<16><<<b.grid(4), kBThreads, 0, b.st>>>(bdev(P), tab, b.T, p, table, slots - 1, bitmap, b.d_status);
    else
        k_bexpand<32><<<b.grid(4), kBThreads, 0, b.st>>>(bdev(P), tab, b.T, p, table, slots - 1, bitmap, b.d_status);
    rc = blaunch(b);
    if (rc) return rc;
    k_bmark<<<b.grid(4), 256, 0, b.st>>>(table, slots, P.child_off, bitmap);
    rc = blaunch(b);
    if (rc) return rc;
    BCK(cudaMemsetAsync(rank + words, 0, 8, b.st));
    k_bpopc<<<b.grid(2), 256, 0, b.st>>>(bitmap, words, rank);
    rc = blaunch(b);
    if (rc) return rc;
    /* each word's rank of kept children, scanned on the device; the kept
       total lands in rank[words] */
    rc = bscan(b, rank, words + 1);
    if (rc) return rc;
    uint64_t kept = 0;
    uint32_t status = 0;
    BCK(cudaMemcpyAsync(&kept, rank + words, 8, cudaMemcpyDeviceToHost, b.st));
    BCK(cudaMemcpyAsync(&status, b.d_status, 4, cudaMemcpyDeviceToHost, b.st));
    BCK(cudaStreamSynchronize(b.st));
    b.d2h += 12;
    if (status) { set_berr("pruning table probe limit reached"); return PCAGB_ELIMIT; }
    rc = alloc_blevel(b, C, kept);
    if (rc) return rc;
    if (kept) {
        if (b.TP == 16)
            k_bmaterialize<16><<<b.grid(4), kBThreads, 0, b.st>>>(bdev(P), tab, b.T, p, bitmap, rank, C);
        else
            k_bmaterialize<32><<<b.grid(4), kBThreads, 0, b.st>>>(bdev(P), tab, b.T, p, bitmap, rank, C);
        rc = blaunch(b);
        if (rc) return rc;
    }
    return PCAGB_OK;
}

/* Host copies of a level's tree links. */
struct HostLevel {
    std::vector<uint32_t> parent;
    std::vector<uint16_t> cidx;
    std::vector<uint8_t> live;
    uint64_t children = 0;
};

int fetch_links(BranchRun &b, const BLevel &L, HostLevel &H, bool links)
{
    H.live.resize(L.n);
    BCK(cudaMemcpyAsync(H.live.data(), L.live, L.n, cudaMemcpyDeviceToHost, b.st));
    b.d2h += L.n;
    if (links) {
        H.parent.resize(L.n);
        H.cidx.resize(L.n);
        BCK(cudaMemcpyAsync(H.parent.data(), L.parent, L.n * 4, cudaMemcpyDeviceToHost, b.st));
        BCK(cudaMemcpyAsync(H.cidx.data(), L.cidx, L.n * 2, cudaMemcpyDeviceToHost, b.st));
        b.d2h += L.n * 6;
    }
    BCK(cudaStreamSynchronize(b.st));
    return PCAGB_OK;
}

/* Kernel words of solutions (state q of level K-1, candidate c) from their
 * tree links, gathered on the device (k_bpath). */
int solution_kernels(BranchRun &b, const BranchTables &bt, std::vector<BLevel> &lv, int K,
                     const std::vector<std::pair<uint32_t, uint16_t>> &sols,
                     std::vector<std::vector<uint16_t>> *kernels)
{
    kernels->clear();
    if (sols.empty()) return PCAGB_OK;
    BPath L{};
    for (int d = 0; d < K; d++) {
        L.parent[d] = lv[d].parent;
        L.cidx[d] = lv[d].cidx;
        L.live[d] = lv[d].live;
    }
    const int ns = (int)sols.size();
    uint32_t *d_q = b.alloc<uint32_t>(ns);
    uint16_t *d_c = b.alloc<uint16_t>(ns);
    uint32_t *d_out = b.alloc<uint32_t>((size_t)ns * K);
    if (!d_q || !d_c || !d_out) { set_berr("device memory exhausted"); return PCAGB_ENOMEM; }
    std::vector<uint32_t> q(ns);
    std::vector<uint16_t> c(ns);
    for (int i = 0; i < ns; i++) {
        q[i] = sols[i].first;
        c[i] = sols[i].second;
    }
    BCK(cudaMemcpyAsync(d_q, q.data(), ns * 4, cudaMemcpyHostToDevice, b.st));
    BCK(cudaMemcpyAsync(d_c, c.data(), ns * 2, cudaMemcpyHostToDevice, b.st));
    k_bpath<<<(ns + 127) / 128, 128, 0, b.st>>>(L, K, d_q, d_c, ns, d_out);
    int rc = blaunch(b);
    if (rc) return rc;
    std::vector<uint32_t> out((size_t)ns * K);
    BCK(cudaMemcpyAsync(out.data(), d_out, out.size() * 4, cudaMemcpyDeviceToHost, b.st));
    BCK(cudaStreamSynchronize(b.st));
    b.h2d += ns * 6;
    b.d2h += out.size() * 4;
    for (int i = 0; i < ns; i++) {
        std::vector<uint16_t> kern(K);
        for (int d = 0; d < K; d++) {
            const uint32_t w = out[(size_t)i * K + d];
            /* position d of a depth-K kernel: forward offsets up to K-d-1 */
            BTab ht{bt.pre_off.data(), bt.post_off.data(), bt.pre.data(), bt.post.data(), K - d - 1};
            kern[d] = bcand(ht, ((w >> 16) >> 1) & 127u, w & 0xFFFFu);
        }
        kernels->push_back(std::move(kern));
    }
    return PCAGB_OK;
}

/* The last position of a depth-K pass without building level K: solving
 * children from k_bsuffix; a child counts only if it is the depth-first
 * first of its key (the pruner would have dropped it otherwise), the
 * smallest child index among k_bsuffix's records with that key, checked by
 * full compares. With first_only the parents are visited in depth-first
 * order in launches of 1/64 of them, doubling, and the search stops at the
 * first launch whose records hold a solution: every child of an earlier
 * launch is earlier in depth-first order, so the records gathered so far
 * settle the first of every key met. Returns the number of solutions found
 * (0 = none at this depth); *searched gets the children of the parents
 * visited. */
int64_t branch_suffix(BranchRun &b, const BranchTables &bt, std::vector<BLevel> &lv, int K,
                      const task_spec_t *task, pcagb_result_t *res, uint16_t *sol_progs,
                      int *sol_lens, int cap, bool first_only, uint64_t *searched)
{
    BLevel &P = lv[K - 1];
    const BTab tab = b.tab(0);
    const uint32_t p = (uint32_t)(K - 1);
    const uint64_t kCap = 1ull << 22;
    BSol *d_sol = b.alloc<BSol>(kCap);
    unsigned long long *d_cnt = b.alloc<unsigned long long>(1);
    if (!d_sol || !d_cnt) { set_berr("device memory exhausted"); return PCAGB_ENOMEM; }
    std::vector<BSol> sol;
    std::vector<size_t> idx;   /* kept solving records, depth-first order */
    uint64_t q0 = 0, step = first_only ? std::max<uint64_t>(P.n / 64, 1) : P.n;
    *searched = 0;
    while (q0 < P.n) {
        const uint64_t q1 = std::min(P.n, q0 + step);
        BCK(cudaMemsetAsync(d_cnt, 0, 8, b.st));
        if (b.TP == 16)
            k_bsuffix<16><<<b.grid(4), kBThreads, 0, b.st>>>(bdev(P), tab, b.T, p, b.d_target,
                                                             d_sol, d_cnt, kCap, q0, q1);
        else
            k_bsuffix<32><<<b.grid(4), kBThreads, 0, b.st>>>(bdev(P), tab, b.T, p, b.d_target,
                                                             d_sol, d_cnt, kCap, q0, q1);
        int rc = blaunch(b);
        if (rc) return rc;
        unsigned long long cnt = 0;
        uint64_t off_end = 0;
        BCK(cudaMemcpyAsync(&cnt, d_cnt, 8, cudaMemcpyDeviceToHost, b.st));
        BCK(cudaMemcpyAsync(&off_end, P.child_off + q1, 8, cudaMemcpyDeviceToHost, b.st));
        BCK(cudaStreamSynchronize(b.st));
        b.d2h += 16;
        *searched = off_end;
        if (cnt > kCap) {
            set_berr("%llu solving children at depth %d: more than the last-position buffer holds",
                     (unsigned long long)cnt, K);
            return PCAGB_ELIMIT;
        }
        q0 = q1;
        step *= 2;
        if (cnt == 0) continue;
        const size_t base = sol.size();
        sol.resize(base + cnt);
        BCK(cudaMemcpyAsync(sol.data() + base, d_sol, cnt * sizeof(BSol), cudaMemcpyDeviceToHost,
                            b.st));
        BCK(cudaStreamSynchronize(b.st));
        b.d2h += cnt * sizeof(BSol);
        bool any = false;
        for (size_t i = base; i < sol.size(); i++) any |= sol[i].mask != 0;
        if (!any) continue;
        /* the depth-first first child of every solving key: the smallest L
           among the records with that key (every child equal to a solving
           one is a record, and no later launch holds a smaller L) */
        std::unordered_map<uint64_t, size_t> first;
        first.reserve(sol.size() * 2);
        for (size_t i = 0; i < sol.size(); i++) {
            auto it = first.find(sol[i].key);
            if (it == first.end()) first.emplace(sol[i].key, i);
            else if (sol[i].L < sol[it->second].L) it->second = i;
        }
        /* a solving child that is not the first of its key is dropped when
           the first is equal to it in full (a 64-bit key collision stops
           here) */
        std::vector<uint4> pairs;
        std::vector<size_t> pair_of;
        std::vector<uint8_t> keep(sol.size(), 0);
        for (size_t i = 0; i < sol.size(); i++) {
            if (!sol[i].mask) continue;
            keep[i] = 1;
            const size_t f = first[sol[i].key];
            if (f == i) continue;
            pairs.push_back(make_uint4(sol[i].q, sol[i].c, sol[f].q, sol[f].c));
            pair_of.push_back(i);
        }
        if (!pairs.empty()) {
            uint4 *d_pairs = b.alloc<uint4>(pairs.size());
            uint8_t *d_eq = b.alloc<uint8_t>(pairs.size());
            if (!d_pairs || !d_eq) { set_berr("device memory exhausted"); return PCAGB_ENOMEM; }
            BCK(cudaMemcpyAsync(d_pairs, pairs.data(), pairs.size() * sizeof(uint4),
                                cudaMemcpyHostToDevice, b.st));
            b.h2d += pairs.size() * sizeof(uint4);
            if (b.TP == 16)
                k_bpairs_equal<16><<<b.grid(2), 256, 0, b.st>>>(bdev(P), tab, b.T, p, d_pairs,
                                                                pairs.size(), d_eq);
            else
                k_bpairs_equal<32><<<b.grid(2), 256, 0, b.st>>>(bdev(P), tab, b.T, p, d_pairs,
                                                                pairs.size(), d_eq);
            rc = blaunch(b);
            if (rc) return rc;
            std::vector<uint8_t> eq(pairs.size());
            BCK(cudaMemcpyAsync(eq.data(), d_eq, pairs.size(), cudaMemcpyDeviceToHost, b.st));
            BCK(cudaStreamSynchronize(b.st));
            b.d2h += pairs.size();
            for (size_t j = 0; j < pairs.size(); j++) {
                if (!eq[j]) {
                    set_berr("64-bit key collision between distinct children at depth %d", K);
                    return PCAGB_ELIMIT;
                }
                keep[pair_of[j]] = 0;
            }
        }
        idx.clear();
        for (size_t i = 0; i < sol.size(); i++)
            if (keep[i]) idx.push_back(i);
        if (!idx.empty() && first_only) break;
    }
    if (idx.empty()) return 0;
    std::sort(idx.begin(), idx.end(), [&](size_t a, size_t c) { return sol[a].L < sol[c].L; });
    /* the reference's walk stops at the leaf that brings its count to 100:
       the (state, register) pairs listed, and the programs of the first cap */
    std::vector<std::pair<uint32_t, uint16_t>> want;
    std::vector<int> want_reg;
    uint64_t listed = 0;
    for (size_t i : idx) {
        for (int r = 1; r < 8; r++) {
            if (!(sol[i].mask >> r & 1u)) continue;
            listed++;
            if ((int)want.size() < cap && sol_progs) {
                want.emplace_back(sol[i].q, sol[i].c);
                want_reg.push_back(r);
            }
        }
        if (listed >= 100) break;
    }
    std::vector<std::vector<uint16_t>> kerns;
    int rc = solution_kernels(b, bt, lv, K, want, &kerns);
    if (rc) return rc;
    int stored = 0;
    for (size_t j = 0; j < kerns.size(); j++) {
        uint16_t prog[16] = {0};
        int n = 0;
        for (int q = 0; q < task->num_inputs; q++)
            prog[n++] = (uint16_t)PCA_ENC_I(PCA_OP_IN, q + 1, task->input_ports[q]);
        for (uint16_t w : kerns[j]) prog[n++] = w;
        prog[n++] = (uint16_t)PCA_ENC_I(PCA_OP_OUT, want_reg[j], task->output_ports[0]);
        prog[n++] = (uint16_t)PCA_ENC_R(PCA_OP_HLT, 0, 0, 0);
        if (task_evaluate(task, prog, n) != task->num_tests) {
            set_berr("internal: a branch-mode solution failed the VM re-check");
            return PCAGB_ELIMIT;
        }
        memcpy(sol_progs + (size_t)stored * 16, prog, sizeof prog);
        if (sol_lens) sol_lens[stored] = n;
        stored++;
    }
    res->stored = stored;
    res->total_solutions = listed;
    return (int64_t)listed;
}

}  // namespace

/* Internal accessors of engine.cu. */
cudaStream_t pcagb_internal_stream(pcagb_engine_t *e);
int pcagb_internal_device(pcagb_engine_t *e);

extern "C" {

const char *pcagb_branch_last_error(void) { return g_berr.c_str(); }

int pcagb_solve_branch(pcagb_engine_t *e, const task_spec_t *task, int max_depth,
                       pcagb_result_t *res, uint16_t *sol_progs, int *sol_lens, int sol_cap)
{
    return pcagb_solve_branch_ex(e, task, max_depth, kMaterializeMax, res, sol_progs, sol_lens,
                                 sol_cap);
}

}  // extern "C"

namespace {

/* Branch-mode IDDFS. first_only: the last position of every depth is
   searched without its level, in depth-first launches that stop at the
   first holding a solution (branch_suffix). */
int solve_branch(pcagb_engine_t *e, const task_spec_t *task, int max_depth,
                 uint64_t last_level_max_children, bool first_only, pcagb_result_t *res,
                 uint16_t *sol_progs, int *sol_lens, int sol_cap)
{
    if (!e || !task || !res) { set_berr("null argument"); return PCAGB_EINVAL; }
    memset(res, 0, sizeof *res);
    res->optimal_depth = -1;
    if (task->num_tests < 1 || task->num_tests > MAX_TESTS || task->num_inputs < 0 ||
        task->num_inputs > 7 || task->num_outputs != 1) {
        set_berr("task needs 1..32 tests, one output and at most 7 inputs");
        return PCAGB_EINVAL;
    }
    if (max_depth < 0 || task->num_inputs + max_depth + 2 > 16) {
        set_berr("max_depth %d out of range (program length is limited to 16)", max_depth);
        return PCAGB_EINVAL;
    }
    if ((uint64_t)task->max_cycles < (uint64_t)(task->num_inputs + max_depth + 2)) {
        set_berr("max_cycles %llu is below the program length", (unsigned long long)task->max_cycles);
        return PCAGB_EINVAL;
    }
    auto t_start = std::chrono::steady_clock::now();
    const BranchTables &bt = branch_tables();
    BranchRun b;
    b.st = pcagb_internal_stream(e);
    BCK(cudaSetDevice(pcagb_internal_device(e)));
    BCK(cudaDeviceGetAttribute(&b.sms, cudaDevAttrMultiProcessorCount, pcagb_internal_device(e)));
    b.task = task;
    b.T = task->num_tests;
    b.TP = b.T <= 16 ? 16 : 32;
    b.d_target = b.alloc<uint32_t>(32);
    b.d_pre_off = b.alloc<uint32_t>(129);
    b.d_post_off = b.alloc<uint32_t>(129);
    b.d_pre = b.alloc<uint16_t>(bt.pre.size());
    b.d_post = b.alloc<uint16_t>(bt.post.size());
    b.d_status = b.alloc<uint32_t>(1);
    if (!b.d_target || !b.d_pre_off || !b.d_post_off || !b.d_pre || !b.d_post || !b.d_status) {
        set_berr("device memory exhausted");
        return PCAGB_ENOMEM;
    }
    uint32_t tgt[32] = {0};
    for (int t = 0; t < b.T; t++) tgt[t] = task->tests[t].out[0];
    BCK(cudaMemcpyAsync(b.d_target, tgt, sizeof tgt, cudaMemcpyHostToDevice, b.st));
    BCK(cudaMemcpyAsync(b.d_pre_off, bt.pre_off.data(), 129 * 4, cudaMemcpyHostToDevice, b.st));
    BCK(cudaMemcpyAsync(b.d_post_off, bt.post_off.data(), 129 * 4, cudaMemcpyHostToDevice, b.st));
    BCK(cudaMemcpyAsync(b.d_pre, bt.pre.data(), bt.pre.size() * 2, cudaMemcpyHostToDevice, b.st));
    BCK(cudaMemcpyAsync(b.d_post, bt.post.data(), bt.post.size() * 2, cudaMemcpyHostToDevice, b.st));

    /* level 0: the IN scaffold's state */
    search_ctx_t ctx;
    if (search_ctx_init(&ctx, task) != 0) { set_berr("bad task"); return PCAGB_EINVAL; }
    search_state_t root;
    search_state_init_root(&ctx, &root);
    std::vector<uint16_t> r0regs((size_t)8 * b.TP, 0);
    std::vector<uint8_t> r0f(b.TP, 0), r0s(b.TP, 0);
    for (int t = 0; t < b.T; t++)
        for (int r = 1; r < 8; r++) r0regs[(size_t)r * b.TP + t] = root.regs[t][r];
    const uint8_t live0 = root.live;
    uint64_t pruned_cum = 0;
    const int cap = std::max(sol_cap, 0);
    const size_t persistent = b.allocs.size();
    for (int K = 0; K <= max_depth; K++) {
        b.release(persistent);  /* the previous depth's levels */
        std::vector<BLevel> lv(K + 1);
        if (alloc_blevel(b, lv[0], 1)) return PCAGB_ENOMEM;
        const uint32_t zero = 0;
        BCK(cudaMemcpyAsync(lv[0].regs, r0regs.data(), r0regs.size() * 2, cudaMemcpyHostToDevice, b.st));
        BCK(cudaMemcpyAsync(lv[0].flags, r0f.data(), b.TP, cudaMemcpyHostToDevice, b.st));
        BCK(cudaMemcpyAsync(lv[0].skip, r0s.data(), b.TP, cudaMemcpyHostToDevice, b.st));
        BCK(cudaMemcpyAsync(lv[0].live, &live0, 1, cudaMemcpyHostToDevice, b.st));
        BCK(cudaMemcpyAsync(lv[0].parent, &zero, 4, cudaMemcpyHostToDevice, b.st));
        BCK(cudaMemcpyAsync(lv[0].cidx, &zero, 2, cudaMemcpyHostToDevice, b.st));
        uint64_t tried = 0, pruned = 0;
        bool unbuilt_last = false;
        for (int d = 0; d < K; d++) {
            const int mf = K - d - 1;
            if (d == K - 1) {
                int rc = count_bchildren(b, lv[d], mf);
                if (rc) return rc;
                if (first_only || lv[d].children > last_level_max_children) {
                    unbuilt_last = true;
                    break;
                }
            }
            int rc = build_blevel(b, lv[d], (uint32_t)d, mf, lv[d + 1]);
            if (rc) return rc;
            tried += lv[d + 1].n;
            pruned += lv[d].children - lv[d + 1].n;
        }
        if (unbuilt_last) {
            /* the engine's counters for this depth: states built plus the
               last position's children (the reference's walk is not
               replayed without the last level) */
            res->split_used = K - 1;
            res->tried[K] = tried + lv[K - 1].children;
            res->pruned_cum[K] = pruned_cum + pruned;
            res->candidates[K] = res->tried[K];
            res->level_children[K] = lv[K - 1].children;
            uint64_t searched = 0;
            const int64_t got = branch_suffix(b, bt, lv, K, task, res, sol_progs, sol_lens, cap,
                                              first_only, &searched);
            if (got < 0) return (int)got;
            if (first_only) {
                res->tried[K] = tried + searched;
                res->candidates[K] = res->tried[K];
            }
            pruned_cum += pruned;
            if (got > 0) {
                res->optimal_depth = K;
                break;
            }
            continue;
        }
        res->level_children[K] = K ? lv[K - 1].children : 1;
        res->level_survivors[K] = lv[K].n;
        /* the output check of every complete kernel */
        const BLevel &LK = lv[K];
        uint8_t *d_mask = b.alloc<uint8_t>(LK.n);
        if (!d_mask) { set_berr("device memory exhausted"); return PCAGB_ENOMEM; }
        if (LK.n) {
            if (b.TP == 16)
                k_bleaf<16><<<b.grid(4), 256, 0, b.st>>>(bdev(LK), b.T, b.d_target, d_mask);
            else
                k_bleaf<32><<<b.grid(4), 256, 0, b.st>>>(bdev(LK), b.T, b.d_target, d_mask);
            int rc = blaunch(b);
            if (rc) return rc;
        }
        std::vector<HostLevel> H(K + 1);
        for (int d = 0; d <= K; d++) {
            int rc = fetch_links(b, lv[d], H[d], d > 0);
            if (rc) return rc;
            H[d].children = lv[d].children;
        }
        std::vector<uint8_t> mask(LK.n);
        BCK(cudaMemcpyAsync(mask.data(), d_mask, LK.n, cudaMemcpyDeviceToHost, b.st));
        BCK(cudaStreamSynchronize(b.st));
        b.d2h += LK.n;
        uint64_t outputs = 0, nsol = 0;
        for (uint64_t i = 0; i < LK.n; i++) {
            outputs += __builtin_popcount(H[K].live[i] >> 1);
            nsol += __builtin_popcount(mask[i]);
        }
        if (nsol == 0) {
            res->tried[K] = tried + outputs;
            pruned_cum += pruned;
            res->pruned_cum[K] = pruned_cum;
            res->candidates[K] = res->tried[K];
            continue;
        }
        /* solutions: the first 100 (state, register) pairs in depth-first
           order; the reference's pass stops there, so its counters are
           those of the depth-first walk up to that leaf */
        const uint64_t kMax = 100;
        std::vector<std::vector<uint64_t>> first(K);
        for (int d = 0; d < K; d++) {
            first[d].assign(lv[d].n + 1, 0);
            for (uint32_t p : H[d + 1].parent) first[d][p + 1]++;
            for (uint64_t i = 0; i < lv[d].n; i++) first[d][i + 1] += first[d][i];
        }
        struct Sol { uint64_t state; int reg; };
        std::vector<Sol> sols;
        uint64_t w_tried = 0, w_pruned = 0;
        bool stop = false;
        auto walk = [&](auto &&self, int d, uint64_t i) -> void {
            if (d == K) {
                const uint32_t live = H[K].live[i];
                w_tried += __builtin_popcount(live >> 1);
                for (int r = 1; r < 8; r++)
                    if (mask[i] >> r & 1u) sols.push_back(Sol{i, r});
                if (sols.size() >= kMax) stop = true;
                return;
            }
            const uint64_t nchild = (d + 1 <= K) ? first[d][i + 1] - first[d][i] : 0;
            const uint32_t m = (H[d].live[i] >> 1) & 127u;
            BTab ht{bt.pre_off.data(), bt.post_off.data(), bt.pre.data(), bt.post.data(), K - d - 1};
            const uint64_t ncand = bcount(ht, m);
            uint64_t seen = 0;
            for (uint64_t j = first[d][i]; j < first[d][i + 1]; j++) {
                /* candidates before this child that it did not visit were pruned */
                w_pruned += H[d + 1].cidx[j] - seen;
                seen = (uint64_t)H[d + 1].cidx[j] + 1;
                w_tried++;
                self(self, d + 1, j);
                if (stop) return;
            }
            (void)nchild;
            w_pruned += ncand - seen;
        };
        walk(walk, 0, 0);
        res->tried[K] = w_tried;
        pruned_cum += w_pruned;
        res->pruned_cum[K] = pruned_cum;
        res->candidates[K] = w_tried;
        res->optimal_depth = K;
        res->total_solutions = sols.size();
        int stored = 0;
        for (const Sol &s : sols) {
            if (stored >= cap || !sol_progs) break;
            std::vector<uint16_t> kern(K);
            uint64_t i = s.state;
            for (int d = K; d >= 1; d--) {
                const uint32_t p = H[d].parent[i];
                BTab ht{bt.pre_off.data(), bt.post_off.data(), bt.pre.data(), bt.post.data(), K - d};
                kern[d - 1] = bcand(ht, (H[d - 1].live[p] >> 1) & 127u, H[d].cidx[i]);
                i = p;
            }
            uint16_t prog[16] = {0};
            int n = 0;
            for (int q = 0; q < task->num_inputs; q++)
                prog[n++] = (uint16_t)PCA_ENC_I(PCA_OP_IN, q + 1, task->input_ports[q]);
            for (uint16_t w : kern) prog[n++] = w;
            prog[n++] = (uint16_t)PCA_ENC_I(PCA_OP_OUT, s.reg, task->output_ports[0]);
            prog[n++] = (uint16_t)PCA_ENC_R(PCA_OP_HLT, 0, 0, 0);
            if (task_evaluate(task, prog, n) != task->num_tests) {
                set_berr("internal: a branch-mode solution failed the VM re-check");
                return PCAGB_ELIMIT;
            }
            memcpy(sol_progs + (size_t)stored * 16, prog, sizeof prog);
            if (sol_lens) sol_lens[stored] = n;
            stored++;
        }
        res->stored = stored;
        break;
    }
    res->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    res->kernel_launches = (uint64_t)b.launches;
    res->h2d_bytes = b.h2d;
    res->d2h_bytes = b.d2h;
    return PCAGB_OK;
}

}  // namespace

extern "C" {

int pcagb_solve_branch_ex(pcagb_engine_t *e, const task_spec_t *task, int max_depth,
                          uint64_t last_level_max_children, pcagb_result_t *res,
                          uint16_t *sol_progs, int *sol_lens, int sol_cap)
{
    return solve_branch(e, task, max_depth, last_level_max_children, false, res, sol_progs,
                        sol_lens, sol_cap);
}

int pcagb_solve_branch_first(pcagb_engine_t *e, const task_spec_t *task, int max_depth,
                             pcagb_result_t *res, uint16_t *sol_progs, int *sol_lens, int sol_cap)
{
    return solve_branch(e, task, max_depth, 0, true, res, sol_progs, sol_lens, sol_cap);
}

}  // extern "C"
