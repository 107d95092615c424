/*
 * valuenet_tc.cu -- the value network's per-test encoder on the fifth-
 * generation tensor cores (tcgen05 + TMEM + TMA), fused from the level's
 * states to the pooled state vector.
 *
 * One persistent CTA per SM walks tiles of 128 feature rows (4 states x 32
 * test rows). Roles: warp 0 streams the weights by TMA (256 x 64 bf16 slabs
 * of W1 then W2, 128-byte swizzle) through a 3-stage ring; warp 1 owns TMEM
 * and one of its threads issues tcgen05.mma (M=128, N=256, K=16, BF16 in,
 * FP32 accumulate); warps 2..17 are the epilogue, four per TMEM lane quarter
 * (one state), each owning 64 of the 256 units. Per tile:
 *   features  the 176 bit features of each (state, test) row (the columns
 *             of k_features in valuenet.cu), expanded to BF16 in registers
 *             straight into the swizzled K-major operand A1;
 *   layer E1  A1 x W1^T into TMEM columns 0..255;
 *   epi 1     tcgen05.ld, + bias, ReLU and BF16 rounding in one packed
 *             convert, into the operand A2 (swizzled, K-major);
 *   layer E2  A2 x W2^T into TMEM columns 256..511;
 *   epi 2     the same on E2's accumulators, written back over the warp's
 *             own part of A2, then pooled: each lane sums (fp32, tests in
 *             order) and maxes (packed bf16) 2 units over the task's T test
 *             rows and writes P[528] = mean(256) | max(256) | live bits(8) |
 *             depth | zeros -- the same values as k_pool on the same H2.
 * A1 and A2 are separate buffers, so the next tile's features and E1 run on
 * the tensor core while the epilogue finishes the current tile's E2.
 * The activations X, H1 and H2 never reach HBM: per state the kernel reads
 * the level record (17 x T bytes) and writes 1,056 bytes; the weights (224
 * KB) are re-read from L2 once per tile.
 *
 * Synchronisation is by mbarriers only; every wait is bounded by the global
 * timer (kWaitNs). A wait that runs out sets the CTA's abort flag and the
 * status word, every role leaves its loop, the producer waits for its own
 * TMA copies, the MMA thread waits for its own MMAs, and TMEM is freed
 * before the CTA returns.
 */
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "../../include/pca_gb300.h"

namespace {

constexpr int kRows = 128;            /* feature rows per tile */
constexpr int kStatesPerTile = 4;
constexpr int kUnits = 256;           /* N of both encoder layers */
constexpr int kFeat = 176;            /* feature columns (164 used) */
constexpr int kKB1 = 3, kKB2 = 4;     /* 64-column K blocks of E1 (176 -> 192) and E2 */
constexpr int kSlabs = kKB1 + kKB2;   /* weight slabs per tile */
constexpr int kStages = 3;
constexpr int kEpiWarps = 16;
constexpr int kEpiThreads = 32 * kEpiWarps;
constexpr int kThreads = 64 + kEpiThreads; /* warp 0 TMA, warp 1 MMA + TMEM, 2..17 epilogue */
constexpr int kABlock = kRows * 128;  /* 16 KB: 128 rows x 64 bf16 */
constexpr int kWBlock = kUnits * 128; /* 32 KB: 256 rows x 64 bf16 */
constexpr int kOffA1 = 0;                             /* 48 KB */
constexpr int kOffA2 = kOffA1 + kKB1 * kABlock;       /* 64 KB */
constexpr int kOffW = kOffA2 + kKB2 * kABlock;        /* 96 KB */
constexpr int kOffBias = kOffW + kStages * kWBlock;   /* 2 x 256 fp32 */
constexpr int kOffBar = kOffBias + 2 * kUnits * 4;
constexpr int kSmemBytes = kOffBar + 256 + 1024;      /* + alignment slack */
constexpr int kPoolCols = 528;
constexpr unsigned long long kWaitNs = 1000000000ull; /* 1 s per wait */
static_assert(kOffA2 % 1024 == 0 && kOffW % 1024 == 0, "swizzle atoms need 1024-byte alignment");
static_assert(kSmemBytes <= 227 * 1024, "shared memory");

/* barrier slots (8 bytes each) */
constexpr int kBarWFull = 0, kBarWEmpty = kStages, kBarA1 = 2 * kStages, kBarA2 = kBarA1 + 1,
              kBarD1 = kBarA1 + 2, kBarD2 = kBarA1 + 3, kBarDrain = kBarA1 + 4,
              kBarCount = kBarA1 + 5;
constexpr int kOffTmemSlot = kBarCount * 8;
constexpr int kOffAbort = kOffTmemSlot + 4;
static_assert(kOffAbort + 4 <= 256, "barrier area");

/* Instruction descriptor of tcgen05.mma kind::f16: D f32 (bits 4-5 = 1),
   A and B bf16 (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bits 17-22,
   M >> 4 at bits 24-28. */
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kUnits >> 3) << 17) |
                            ((uint32_t)(kRows >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_test(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

/* Wait for the phase of `parity` to complete, at most kWaitNs; on time-out
   (or an abort raised elsewhere) set the abort flag and return false. */
__device__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int *abort_flag, int *status,
                          int code)
{
    const unsigned long long t0 = global_ns();
    for (uint32_t i = 0;; i++) {
        if (mbar_test(bar, parity)) return true;
        if ((i & 15) == 15) {
            if (*abort_flag) return false;
            if (global_ns() - t0 > kWaitNs) {
                *abort_flag = 1;
                atomicExch(status, code);
                return false;
            }
        }
    }
}

__device__ __forceinline__ void fence_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void tc_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, uint32_t bar,
                                            int x, int y)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%3, %4}], [%2];" ::"r"(dst),
        "l"((uint64_t)map), "r"(bar), "r"(x), "r"(y)
        : "memory");
}

/* Shared-memory matrix descriptor: K-major operand in 128-byte swizzle
   atoms (8 rows x 128 B), 8-row groups 1024 B apart. */
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr)
{
    uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;            /* leading byte offset: unused for swizzled K-major */
    d |= (uint64_t)(1024 >> 4) << 32;  /* stride byte offset */
    d |= (uint64_t)1 << 46;            /* descriptor version */
    d |= (uint64_t)2 << 61;            /* 128-byte swizzle */
    return d;
}

/* Shared-memory matrix descriptor: MN-major operand in 128-byte swizzle
   atoms (8 K-rows x 128 B = 64 elements along M or N), 8-row groups 1024 B
   apart along K, 64-element groups along M or N 8 KB apart (one 64 x 64
   TMA box each). */
__device__ __forceinline__ uint64_t sw128_mn_desc(uint32_t saddr)
{
    uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)(8192 >> 4) << 16;  /* leading byte offset: next 64 along M/N */
    d |= (uint64_t)(1024 >> 4) << 32;  /* stride byte offset: next 8 along K */
    d |= (uint64_t)1 << 46;            /* descriptor version */
    d |= (uint64_t)2 << 61;            /* 128-byte swizzle */
    return d;
}

__device__ __forceinline__ void mma_f16(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
        "l"(a), "l"(b), "r"(kIdesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar)
{
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
        : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32])
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
          "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
          "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

/* Byte offset of 16-byte chunk c (0..7) of row r in a 128-byte-swizzled
   block (the layout TMA's 128B swizzle writes and the descriptor reads). */
__device__ __forceinline__ uint32_t sw128_off(int r, int c)
{
    return (uint32_t)(r * 128 + ((c ^ (r & 7)) << 4));
}

/* 8 bits of b as 8 bf16 values 0.0 / 1.0 (bit 0 first): bit 2j selects
   0x3F80 in the low half of word j, bit 2j+1 0x3F80 in the high half. */
__device__ __forceinline__ uint4 bits_to_bf16x8(uint32_t b)
{
    uint32_t w[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const uint32_t t = b >> (2 * j);
        w[j] = (t & 1u) * 0x3F80u + (t & 2u) * 0x1FC00000u;
    }
    return make_uint4(w[0], w[1], w[2], w[3]);
}

/* relu(lo), relu(hi) rounded to bf16, lo in the low half. */
__device__ __forceinline__ uint32_t relu_bf16x2(float lo, float hi)
{
    uint32_t d;
    asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
    return d;
}

__device__ __forceinline__ uint32_t max_bf16x2(uint32_t a, uint32_t b)
{
    uint32_t d;
    asm("max.bf16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
    return d;
}

__global__ void __launch_bounds__(kThreads, 1)
k_encode_pool_tc(const __grid_constant__ CUtensorMap map_w1, const __grid_constant__ CUtensorMap map_w2,
                 const float *__restrict__ b1, const float *__restrict__ b2,
                 const uint16_t *__restrict__ regs, const uint8_t *__restrict__ flags,
                 const uint8_t *__restrict__ live, const uint16_t *__restrict__ task,
                 const uint8_t *__restrict__ depth, int TP, int n,
                 const uint16_t *__restrict__ task_io, const int32_t *__restrict__ task_T,
                 __nv_bfloat16 *__restrict__ P, int *status)
{
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const uint32_t sA1 = smem_u32(smem + kOffA1), sA2 = smem_u32(smem + kOffA2);
    const uint32_t sW = smem_u32(smem + kOffW);
    const uint32_t sBar = smem_u32(smem + kOffBar);
    uint32_t *tmem_slot = (uint32_t *)(smem + kOffBar + kOffTmemSlot);
    volatile int *abort_flag = (volatile int *)(smem + kOffBar + kOffAbort);
    float *sb1 = (float *)(smem + kOffBias);
    float *sb2 = sb1 + kUnits;
    auto bar = [&](int i) { return sBar + 8u * (uint32_t)i; };

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ntiles = (n + kStatesPerTile - 1) / kStatesPerTile;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; s++) {
            mbar_init(bar(kBarWFull + s), 1);
            mbar_init(bar(kBarWEmpty + s), 1);
        }
        mbar_init(bar(kBarA1), kEpiThreads);
        mbar_init(bar(kBarA2), kEpiThreads);
        mbar_init(bar(kBarD1), 1);
        mbar_init(bar(kBarD2), 1);
        mbar_init(bar(kBarDrain), 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        fence_async_smem();
    }
    for (int i = threadIdx.x; i < kUnits; i += kThreads) {
        sb1[i] = b1[i];
        sb2[i] = b2[i];
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(
                         smem_u32(tmem_slot))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_before();
    __syncthreads();
    tc_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        /* ---- TMA producer: weight slabs through the ring ---- */
        if (lane == 0) {
            uint32_t j = 0;
            bool ok = true;
            for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
                for (int s = 0; s < kSlabs && ok; s++, j++) {
                    const uint32_t st = j % kStages, ph = (j / kStages) & 1u;
                    ok = mbar_wait(bar(kBarWEmpty + st), ph ^ 1u, abort_flag, status, 1);
                    if (!ok) break;
                    mbar_expect_tx(bar(kBarWFull + st), kWBlock);
                    if (s < kKB1)
                        tma_load_2d(sW + st * kWBlock, &map_w1, bar(kBarWFull + st), s * 64, 0);
                    else
                        tma_load_2d(sW + st * kWBlock, &map_w2, bar(kBarWFull + st),
                                    (s - kKB1) * 64, 0);
                }
            }
            /* wait for the copies this thread issued (the last one per stage) */
            const uint32_t issued = j;
            for (uint32_t st = 0; st < kStages && st < issued; st++) {
                const uint32_t last = issued - 1 - ((issued - 1 - st) % kStages);
                const unsigned long long t0 = global_ns();
                while (!mbar_test(bar(kBarWFull + st), (last / kStages) & 1u) &&
                       global_ns() - t0 < kWaitNs) {
                }
            }
        }
    } else if (warp == 1) {
        /* ---- MMA issuer ---- */
        if (lane == 0) {
            uint32_t j = 0;
            bool ok = true;
            int it = 0;
            for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x, it++) {
                for (int layer = 0; layer < 2 && ok; layer++) {
                    ok = mbar_wait(bar(layer ? kBarA2 : kBarA1), it & 1, abort_flag, status, 2);
                    if (!ok) break;
                    tc_after();
                    const int nkb = layer ? kKB2 : kKB1;
                    const uint32_t d = tmem + (layer ? (uint32_t)kUnits : 0u);
                    const uint32_t a = layer ? sA2 : sA1;
                    for (int kb = 0; kb < nkb; kb++, j++) {
                        const uint32_t st = j % kStages, ph = (j / kStages) & 1u;
                        ok = mbar_wait(bar(kBarWFull + st), ph, abort_flag, status, 3);
                        if (!ok) break;
                        tc_after();
                        const uint32_t a0 = a + kb * kABlock, b0 = sW + st * kWBlock;
#pragma unroll
                        for (int k = 0; k < 4; k++)
                            mma_f16(d, sw128_desc(a0 + 32 * k), sw128_desc(b0 + 32 * k),
                                    (kb | k) != 0);
                        mma_commit(bar(kBarWEmpty + st));
                    }
                    if (!ok) break;
                    mma_commit(bar(layer ? kBarD2 : kBarD1));
                }
            }
            /* every MMA this thread issued has finished before TMEM is freed */
            mma_commit(bar(kBarDrain));
            const unsigned long long t0 = global_ns();
            while (!mbar_test(bar(kBarDrain), 0) && global_ns() - t0 < kWaitNs) {
            }
        }
    } else {
        /* ---- epilogue warps ---- */
        const int q = warp & 3;              /* TMEM lane quarter = the tile's state */
        const int h = (warp - 2) >> 2;       /* units [64h, 64h + 64) */
        const int r = q * 32 + lane;         /* tile row = TMEM lane */
        const uint32_t lane_base = (uint32_t)(q * 32) << 16;

        /* A state's level record, loaded one tile ahead of its features:
           the three 16-bit words of this warp's quarter of the feature row
           (h = 0: in0 in1 target; 1: r1 r2 r3; 2: r4 r5 r6; 3: r7 flags 0)
           for test `lane`, the task's T and (h = 0, lanes 0..15) the pooled
           row's tail. The task id is loaded a tile earlier still, so no
           load waits on another in the loop. */
        struct Rec {
            int s, T;
            uint32_t w[3];
            float g;  /* P column 512 + lane: live bit / depth / 0 */
        };
        auto task_of = [&](int tile) -> int {
            const int st = tile * kStatesPerTile + q;
            return (tile < ntiles && st < n) ? (int)task[st] : -1;
        };
        auto load_rec = [&](int tile, int tid, Rec &rc) {
            rc.s = tile * kStatesPerTile + q;
            rc.T = 0;
            rc.g = 0.f;
            rc.w[0] = rc.w[1] = rc.w[2] = 0;
            if (tid < 0) return;
            rc.T = min(task_T[tid], TP);
            if (h == 0 && lane < 8) rc.g = (float)((live[rc.s] >> lane) & 1u);
            else if (h == 0 && lane == 8) rc.g = (float)depth[rc.s];
            if (lane >= TP) return;
            const size_t s8 = (size_t)rc.s * 8;
            if (h == 0) {
#pragma unroll
                for (int k = 0; k < 3; k++) rc.w[k] = task_io[((size_t)tid * 3 + k) * 32 + lane];
            } else if (h < 3) {
#pragma unroll
                for (int k = 0; k < 3; k++) rc.w[k] = regs[(s8 + 3 * h - 2 + k) * TP + lane];
            } else {
                rc.w[0] = regs[(s8 + 7) * TP + lane];
                rc.w[1] = flags[(size_t)rc.s * TP + lane] & 0xFu;
            }
        };
        /* bit features of (state, test lane), chunks [6h, 6h + 6) of the
           row's 24 16-byte chunks, into A1 (rows of tests >= T are zero) */
        auto features = [&](const Rec &rc) {
            const bool valid = lane < rc.T;
#pragma unroll
            for (int k = 0; k < 6; k++) {
                const int c = 6 * h + k;
                const uint32_t byte = valid ? (rc.w[k >> 1] >> ((k & 1) * 8)) & 0xFFu : 0u;
                *(uint4 *)(smem + kOffA1 + (c >> 3) * kABlock + sw128_off(r, c & 7)) =
                    bits_to_bf16x8(byte);
            }
            fence_async_smem();
            mbar_arrive(bar(kBarA1));
        };

        /* accumulators of units [64h, 64h + 64) of one layer: + bias, ReLU,
           bf16, into this warp's part of A2 */
        auto drain = [&](uint32_t col_base, const float *bias) {
#pragma unroll 1
            for (int g = 0; g < 2; g++) {
            const int col0 = 64 * h + 32 * g;
            uint32_t acc[32];
            tmem_ld32(tmem + col_base + lane_base + col0, acc);
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const float4 bl = *(const float4 *)(bias + col0 + 8 * c);
                const float4 bh = *(const float4 *)(bias + col0 + 8 * c + 4);
                const uint32_t *a = acc + 8 * c;
                const uint32_t w0 = relu_bf16x2(__uint_as_float(a[0]) + bl.x, __uint_as_float(a[1]) + bl.y);
                const uint32_t w1 = relu_bf16x2(__uint_as_float(a[2]) + bl.z, __uint_as_float(a[3]) + bl.w);
                const uint32_t w2 = relu_bf16x2(__uint_as_float(a[4]) + bh.x, __uint_as_float(a[5]) + bh.y);
                const uint32_t w3 = relu_bf16x2(__uint_as_float(a[6]) + bh.z, __uint_as_float(a[7]) + bh.w);
                const int chunk = (col0 >> 3) + c;
                *(uint4 *)(smem + kOffA2 + (chunk >> 3) * kABlock + sw128_off(r, chunk & 7)) =
                    make_uint4(w0, w1, w2, w3);
            }
            }
        };

        /* mean (fp32 over tests in order, as k_pool) and max of units
           64h + 2 lane, + 1 over the state's T rows of H2 in A2 */
        auto pool = [&](const Rec &rc) {
            const int chunk = 8 * h + (lane >> 2);
            const uint8_t *base = smem + kOffA2 + (chunk >> 3) * kABlock + ((lane & 3) << 2);
            float s0 = 0.f, s1 = 0.f;
            uint32_t m01 = 0u;                /* ReLU outputs are >= 0 */
            for (int t0 = 0; t0 < rc.T; t0 += 8) {
                uint32_t v[8];
#pragma unroll
                for (int k = 0; k < 8; k++)
                    v[k] = *(const uint32_t *)(base + sw128_off(32 * q + t0 + k, chunk & 7));
                const bool full = t0 + 8 <= rc.T;
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    const uint32_t x = (full || t0 + k < rc.T) ? v[k] : 0u;
                    s0 += __uint_as_float(x << 16);
                    s1 += __uint_as_float(x & 0xFFFF0000u);
                    m01 = max_bf16x2(m01, x);
                }
            }
            const float fT = (float)(rc.T > 0 ? rc.T : 1);
            __nv_bfloat162 mean = __floats2bfloat162_rn(s0 / fT, s1 / fT);
            __nv_bfloat16 *row = P + (size_t)rc.s * kPoolCols;
            *(uint32_t *)(row + 64 * h + 2 * lane) = *reinterpret_cast<uint32_t *>(&mean);
            *(uint32_t *)(row + kUnits + 64 * h + 2 * lane) = m01;
            if (h == 0 && lane < 16) row[2 * kUnits + lane] = __float2bfloat16(rc.g);
        };

        const int G = (int)gridDim.x;
        int it = 0;
        int tile = blockIdx.x;
        Rec cur, nxt;
        load_rec(tile, task_of(tile), cur);
        int tid_next = task_of(tile + G);
        if (tile < ntiles) features(cur);
        for (; tile < ntiles; tile += G, it++) {
            /* the next tile's record, in flight while E1 drains */
            load_rec(tile + G, tid_next, nxt);
            tid_next = task_of(tile + 2 * G);
            /* E1 -> A2 */
            bool ok = mbar_wait(bar(kBarD1), it & 1, abort_flag, status, 4);
            if (!__all_sync(0xffffffffu, ok)) break;
            tc_after();
            drain(0u, sb1);
            tc_before();
            fence_async_smem();
            mbar_arrive(bar(kBarA2));
            /* next tile's features while E2 runs */
            if (tile + G < ntiles) features(nxt);
            /* E2 -> H2 (over this warp's part of A2) -> pooling */
            ok = mbar_wait(bar(kBarD2), it & 1, abort_flag, status, 5);
            if (!__all_sync(0xffffffffu, ok)) break;
            tc_after();
            drain((uint32_t)kUnits, sb2);
            tc_before();
            __syncwarp();
            if (cur.s < n) pool(cur);
            __syncwarp();
            cur = nxt;
        }
    }
    __syncwarp();
    tc_before();
    __syncthreads();
    tc_after();
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem)
                     : "memory");
}

/* ---- the training GEMM ------------------------------------------------------
 *
 * C[M,N] = A[M,K] . B[N,K]^T on tcgen05, both operands K-major bf16 in HBM,
 * FP32 accumulation in TMEM. One CTA per 128 x bn tile of C (bn <= 256, a
 * multiple of 16), grid.z splits K. Warp 0 (one thread) streams 64-column K
 * blocks of A (128 rows) and B (bn rows) by TMA with 128-byte swizzle
 * through a two-stage mbarrier ring; warp 1 owns TMEM and one thread issues
 * four tcgen05.mma (M=128, N=bn, K=16) per block; then all four warps drain
 * the accumulators (warp w: TMEM lanes 32w..32w+31 = tile rows) with
 * tcgen05.ld. Epilogue: with one K split, + bias, x (mask > 0) (the ReLU
 * derivative through a stored activation), ReLU, stored as bf16 or fp32;
 * with several, fp32 atomic adds into C (zeroed by the caller). Out-of-range
 * rows and columns of A and B are TMA zero fill; stores are bounds checked.
 * Every wait is bounded by the global timer; a wait that runs out sets the
 * abort flag and *status, each role leaves, and TMEM is freed. Two CTAs fit
 * an SM (96 KB of shared memory at bn = 256), so one CTA's epilogue overlaps
 * the other's loads and MMAs.
 *
 * mn_major: A and B are given K-row by K-row instead ([K][M] and [K][N],
 * M and N contiguous: the weight gradient dY^T . X reads dY [batch][out]
 * and X [batch][in] as stored), loaded as 64 x 64 boxes (64 K-rows of 64
 * elements along M or N) and described to the MMA as MN-major operands;
 * bn is then a multiple of 64. */
constexpr int kGRows = 128, kGBK = 64, kGStages = 2;
constexpr int kGABytes = kGRows * 128;              /* 16 KB per A stage */

__global__ void __launch_bounds__(128, 2)
k_gemm_tc(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b,
          const float *__restrict__ bias, const __nv_bfloat16 *__restrict__ mask, int ldm,
          __nv_bfloat16 *__restrict__ Cb, float *__restrict__ Cf, int ldc, int M, int N,
          int kblocks, int kb_per_split, int bn, uint32_t idesc, uint32_t tmem_cols, int relu,
          int atomic_out, int stage_mode, int vec_atomic, int mn_major, int *status)
{
    extern __shared__ uint8_t gsmem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)gsmem_raw + 1023) & ~(uintptr_t)1023);
    const uint32_t b_bytes = (uint32_t)bn * 128u;
    const uint32_t sA = smem_u32(smem);
    const uint32_t sB = sA + kGStages * kGABytes;
    uint8_t *ctl = smem + kGStages * (kGABytes + b_bytes);
    const uint32_t sBar = smem_u32(ctl);
    uint32_t *tmem_slot = (uint32_t *)(ctl + 64);
    volatile int *abort_flag = (volatile int *)(ctl + 68);
    auto full = [&](int s) { return sBar + 8u * (uint32_t)s; };
    auto empty = [&](int s) { return sBar + 8u * (uint32_t)(kGStages + s); };
    const uint32_t done_bar = sBar + 8u * (uint32_t)(2 * kGStages);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.y * kGRows, n0 = blockIdx.x * bn;
    const int kb0 = blockIdx.z * kb_per_split;
    const int nk = min(kblocks, kb0 + kb_per_split) - kb0;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kGStages; s++) {
            mbar_init(full(s), 1);
            mbar_init(empty(s), 1);
        }
        mbar_init(done_bar, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        fence_async_smem();
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tmem_slot)), "r"(tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_before();
    __syncthreads();
    tc_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0 && lane == 0 && nk > 0) {
        /* producer */
        int i = 0;
        for (; i < nk; i++) {
            const int st = i % kGStages;
            const uint32_t ph = (uint32_t)(i / kGStages) & 1u;
            if (!mbar_wait(empty(st), ph ^ 1u, abort_flag, status, 11)) break;
            mbar_expect_tx(full(st), kGABytes + b_bytes);
            const int x = (kb0 + i) * kGBK;
            if (mn_major) {
                /* boxes of 64 K-rows x 64 columns, 8 KB each */
                for (int h = 0; h < kGRows / 64; h++)
                    tma_load_2d(sA + st * kGABytes + h * 8192, &map_a, full(st), m0 + 64 * h, x);
                for (int h = 0; h < bn / 64; h++)
                    tma_load_2d(sB + st * b_bytes + h * 8192, &map_b, full(st), n0 + 64 * h, x);
            } else {
                tma_load_2d(sA + st * kGABytes, &map_a, full(st), x, m0);
                tma_load_2d(sB + st * b_bytes, &map_b, full(st), x, n0);
            }
        }
        /* the copies this thread issued land before the CTA leaves */
        for (int j = i - 1; j >= 0 && j >= i - kGStages; j--) {
            const unsigned long long t0 = global_ns();
            while (!mbar_test(full(j % kGStages), (uint32_t)(j / kGStages) & 1u) &&
                   global_ns() - t0 < kWaitNs) {
            }
        }
    } else if (warp == 1 && lane == 0) {
        /* MMA issuer */
        for (int i = 0; i < nk; i++) {
            const int st = i % kGStages;
            const uint32_t ph = (uint32_t)(i / kGStages) & 1u;
            if (!mbar_wait(full(st), ph, abort_flag, status, 12)) break;
            tc_after();
            const uint32_t a0 = sA + st * kGABytes, b0 = sB + st * b_bytes;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                /* 16 K per MMA: 32 bytes along a K-major row, or two 8-row
                   groups (2 KB) of an MN-major box */
                const uint64_t da = mn_major ? sw128_mn_desc(a0 + 2048 * k) : sw128_desc(a0 + 32 * k);
                const uint64_t db = mn_major ? sw128_mn_desc(b0 + 2048 * k) : sw128_desc(b0 + 32 * k);
                const uint32_t acc = (i | k) != 0;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                    "l"(da), "l"(db), "r"(idesc), "r"(acc)
                    : "memory");
            }
            mma_commit(empty(st));
        }
        /* arrives once every MMA above has completed (also after an abort);
           this thread waits for it, so TMEM is never freed under an MMA */
        mma_commit(done_bar);
        const unsigned long long t0 = global_ns();
        while (!mbar_test(done_bar, 0) && global_ns() - t0 < kWaitNs) {
        }
    }
    __syncwarp();
    /* epilogue: all four warps. The tile's bias goes to shared memory
       first (every thread takes part, so the barrier below is reached by
       all of them whatever the waits return). */
    float *sbias = (float *)(ctl + 256);
    for (int c = threadIdx.x; c < bn; c += 128) sbias[c] = (bias && n0 + c < N) ? bias[n0 + c] : 0.f;
    bool ok = nk > 0 && mbar_wait(done_bar, 0, abort_flag, status, 13);
    ok = __all_sync(0xFFFFFFFFu, ok) && !*abort_flag;
    tc_after();
    __syncthreads();
    if (ok && stage_mode) {
        /* Staged: each warp drains its 32 rows of accumulators (+ bias,
           ReLU, rounding) into the drained stage buffers, a row of bn values
           at a stride of one row + 16 bytes (16-byte stores of eight lanes
           fall on distinct bank groups), then writes its rows to C in
           16-byte pieces, lanes along a row (coalesced), applying the mask
           on the way. stage_mode 1: bf16 C; 2: fp32 C (bn <= 112). */
        const int esz = stage_mode == 1 ? 2 : 4;
        const uint32_t S = (uint32_t)(bn * esz + 16);
        const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
        uint8_t *myrow = smem + (uint32_t)(warp * 32 + lane) * S;
        for (int c0 = 0; c0 < bn; c0 += 32) {
            uint32_t acc[32];
            tmem_ld32(tmem + lane_base + (uint32_t)c0, acc);
            if (stage_mode == 1) {
                uint32_t w[16];
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    const float v0 = __uint_as_float(acc[2 * j]) + sbias[c0 + 2 * j];
                    const float v1 = __uint_as_float(acc[2 * j + 1]) + sbias[c0 + 2 * j + 1];
                    if (relu) {
                        w[j] = relu_bf16x2(v0, v1);
                    } else {
                        __nv_bfloat162 h = __floats2bfloat162_rn(v0, v1);
                        w[j] = *reinterpret_cast<uint32_t *>(&h);
                    }
                }
                /* the tile may end inside this group of 32 (bn = 16) */
#pragma unroll
                for (int k = 0; k < 4; k++)
                    if (c0 + 8 * k < bn)
                        *(uint4 *)(myrow + c0 * 2 + 16 * k) =
                            make_uint4(w[4 * k], w[4 * k + 1], w[4 * k + 2], w[4 * k + 3]);
            } else {
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    float v[4];
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        v[q] = __uint_as_float(acc[4 * k + q]) + sbias[c0 + 4 * k + q];
                        if (relu) v[q] = fmaxf(v[q], 0.f);
                    }
                    if (c0 + 4 * k < bn)
                        *(float4 *)(myrow + c0 * 4 + 16 * k) = make_float4(v[0], v[1], v[2], v[3]);
                }
            }
        }
        __syncwarp();
        const int per = 16 / esz;                 /* values per 16-byte piece */
        const int cpr = bn / per;                 /* pieces per row */
        /* the mask's pieces of four iterations are loaded before any of
           them is used, so each lane has four global loads in flight */
        uint4 mkq[4];
        for (int it = lane; it < 32 * cpr; it += 32) {
            const int u = ((it - lane) >> 5) & 3;
            if (stage_mode == 1 && mask && u == 0) {
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const int itk = it + 32 * k;
                    const int rk = itk / cpr, gr = m0 + warp * 32 + rk;
                    const int gc = n0 + (itk - rk * cpr) * per;
                    mkq[k] = itk < 32 * cpr && gr < M && gc < N
                                 ? *(const uint4 *)(mask + (size_t)gr * ldm + gc)
                                 : make_uint4(0u, 0u, 0u, 0u);
                }
            }
            const int r = it / cpr, ch = it - r * cpr;
            const int grow = m0 + warp * 32 + r, gcol = n0 + ch * per;
            if (grow >= M || gcol >= N) continue;
            const uint8_t *src = smem + (uint32_t)(warp * 32 + r) * S + ch * 16;
            if (stage_mode == 1) {
                uint4 v = *(const uint4 *)src;
                if (mask) {
                    uint4 mk = mkq[0];
#pragma unroll
                    for (int k = 1; k < 4; k++)
                        if (u == k) mk = mkq[k];
                    /* keep a value where its mask half is a positive bf16 */
                    auto keep = [](uint32_t m) {
                        return (__uint_as_float(m << 16) > 0.f ? 0x0000FFFFu : 0u) |
                               (__uint_as_float(m & 0xFFFF0000u) > 0.f ? 0xFFFF0000u : 0u);
                    };
                    v.x &= keep(mk.x);
                    v.y &= keep(mk.y);
                    v.z &= keep(mk.z);
                    v.w &= keep(mk.w);
                }
                if (gcol + per <= N) {
                    *(uint4 *)(Cb + (size_t)grow * ldc + gcol) = v;
                } else {
                    const uint32_t w4[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                    for (int q = 0; q < 8; q++)
                        if (gcol + q < N) {
                            const uint32_t b = (w4[q >> 1] >> (16 * (q & 1))) & 0xFFFFu;
                            reinterpret_cast<uint16_t *>(Cb)[(size_t)grow * ldc + gcol + q] =
                                (uint16_t)b;
                        }
                }
            } else {
                const float4 v = *(const float4 *)src;
                if (gcol + per <= N) {
                    *(float4 *)(Cf + (size_t)grow * ldc + gcol) = v;
                } else {
                    const float f4[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                    for (int q = 0; q < 4; q++)
                        if (gcol + q < N) Cf[(size_t)grow * ldc + gcol + q] = f4[q];
                }
            }
        }
    } else if (ok) {
        /* direct: split-K partial sums (fp32 adds, four at a time where
           aligned) or outputs the staged forms do not cover */
        const int row = m0 + warp * 32 + lane;
        const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
        for (int c0 = 0; c0 < bn; c0 += 32) {
            uint32_t acc[32];
            tmem_ld32(tmem + lane_base + (uint32_t)c0, acc);
            if (row >= M) continue;
            const int colb = n0 + c0;
            if (atomic_out == 2) {
                /* this K split's own slab: plain stores, summed later in
                   split order (deterministic) */
                float *dst = Cf + ((size_t)blockIdx.z * M + row) * ldc + colb;
#pragma unroll
                for (int j = 0; j < 32; j += 4) {
                    if (vec_atomic && colb + j + 3 < N) {
                        *(float4 *)(dst + j) =
                            make_float4(__uint_as_float(acc[j]), __uint_as_float(acc[j + 1]),
                                        __uint_as_float(acc[j + 2]), __uint_as_float(acc[j + 3]));
                    } else {
#pragma unroll
                        for (int q = 0; q < 4; q++)
                            if (colb + j + q < N) dst[j + q] = __uint_as_float(acc[j + q]);
                    }
                }
                continue;
            }
            if (atomic_out) {
                float *dst = Cf + (size_t)row * ldc + colb;
#pragma unroll
                for (int j = 0; j < 32; j += 4) {
                    if (vec_atomic && colb + j + 3 < N) {
                        atomicAdd((float4 *)(dst + j),
                                  make_float4(__uint_as_float(acc[j]), __uint_as_float(acc[j + 1]),
                                              __uint_as_float(acc[j + 2]), __uint_as_float(acc[j + 3])));
                    } else {
#pragma unroll
                        for (int q = 0; q < 4; q++)
                            if (colb + j + q < N) atomicAdd(dst + j + q, __uint_as_float(acc[j + q]));
                    }
                }
                continue;
            }
#pragma unroll
            for (int j = 0; j < 32; j += 2) {
                const int c = colb + j;
                if (c >= N) continue;
                float v0 = __uint_as_float(acc[j]) + sbias[c0 + j];
                float v1 = __uint_as_float(acc[j + 1]) + sbias[c0 + j + 1];
                if (mask) {
                    const __nv_bfloat16 *mr = mask + (size_t)row * ldm + c;
                    if (!(__bfloat162float(mr[0]) > 0.f)) v0 = 0.f;
                    if (c + 1 < N && !(__bfloat162float(mr[1]) > 0.f)) v1 = 0.f;
                }
                if (relu) {
                    v0 = fmaxf(v0, 0.f);
                    v1 = fmaxf(v1, 0.f);
                }
                if (Cb) {
                    if (c + 1 < N)
                        *(__nv_bfloat162 *)(Cb + (size_t)row * ldc + c) = __floats2bfloat162_rn(v0, v1);
                    else
                        Cb[(size_t)row * ldc + c] = __float2bfloat16(v0);
                }
                if (Cf) {
                    Cf[(size_t)row * ldc + c] = v0;
                    if (c + 1 < N) Cf[(size_t)row * ldc + c + 1] = v1;
                }
            }
        }
    }
    tc_before();
    __syncthreads();
    tc_after();
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(tmem_cols)
                     : "memory");
}


typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn()
{
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
    });
    return fn;
}

/* Tensor map of a row-major [256][K] bf16 weight, 64 x 256 boxes, 128B swizzle. */
bool weight_map(CUtensorMap *m, const void *W, int K)
{
    EncodeTiledFn fn = encode_fn();
    if (!fn) return false;
    cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)kUnits};
    cuuint64_t strides[1] = {(cuuint64_t)K * 2};
    cuuint32_t box[2] = {64, (cuuint32_t)kUnits};
    cuuint32_t estr[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(W), dims, strides, box,
              estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
              CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

/* Tensor map of a row-major [rows][cols] bf16 matrix (row stride ld
   elements), boxes of 64 columns x box_rows rows, 128-byte swizzle. */
bool tile_map(CUtensorMap *m, const void *ptr, int rows, int cols, int ld, int box_rows)
{
    EncodeTiledFn fn = encode_fn();
    if (!fn) return false;
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    cuuint32_t box[2] = {64, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(ptr), dims, strides, box,
              estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
              CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

/* C[M,N] = A[M,K] . B[N,K]^T on tcgen05 (k_gemm_tc): bias[N] added, then
 * columns where mask[M][N] (bf16, leading dimension ldm) is not positive
 * zeroed, then ReLU, into Cb (bf16) and/or Cf (fp32), leading dimension ldc.
 * splits > 1 divides K among CTAs that add fp32 partial sums into Cf (zeroed
 * by the caller; no bias, mask, ReLU or Cb then). A and B: leading
 * dimensions multiples of 8 elements, 16-byte aligned. *status gets a
 * nonzero code if a barrier wait ran out (the result is then void). */
extern "C" int pcagb_vnet_gemm_tc(const void *A, int lda, const void *B, int ldb,
                                  const float *bias, const void *mask, int ldm, void *Cb,
                                  float *Cf, int ldc, int M, int N, int K, int relu, int splits,
                                  int *status, void *stream)
{
    if (M <= 0 || N <= 0 || K <= 0) return PCAGB_OK;
    if (!A || !B || !status || (!Cb && !Cf) || (lda & 7) || (ldb & 7) || lda < K || ldb < K ||
        ((uintptr_t)A & 15) || ((uintptr_t)B & 15) || splits < 1 ||
        (splits > 1 && (!Cf || Cb || bias || mask || relu)))
        return PCAGB_EINVAL;
    const int bn = N > 256 ? 256 : (N + 15) / 16 * 16;
    uint32_t tcols = 32;
    while (tcols < (uint32_t)bn) tcols <<= 1;
    CUtensorMap ma, mb;
    if (!tile_map(&ma, A, M, K, lda, kGRows) || !tile_map(&mb, B, N, K, ldb, bn))
        return PCAGB_ECUDA;
    const int kblocks = (K + kGBK - 1) / kGBK;
    if (splits > kblocks) splits = kblocks;
    const int per = (kblocks + splits - 1) / splits;
    splits = (kblocks + per - 1) / per;
    const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(bn >> 3) << 17) |
                           ((uint32_t)(kGRows >> 4) << 24);
    /* stage buffers, then 256 bytes of barriers and flags, the tile's bias
       (bn floats), 1 KB of alignment slack */
    const int smem = kGStages * (kGABytes + bn * 128) + 256 + 1024 + 1024;
    static std::once_flag attr_once;
    static cudaError_t attr_err = cudaSuccess;
    std::call_once(attr_once, [] {
        attr_err = cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        kGStages * (kGABytes + 256 * 128) + 256 + 2048);
    });
    /* the epilogue: staged through shared memory and stored in 16-byte
       pieces where the output's alignment allows */
    int stage_mode = 0;
    if (splits == 1 && Cb && !Cf && ldc % 8 == 0 && !((uintptr_t)Cb & 15) &&
        (!mask || (ldm % 8 == 0 && !((uintptr_t)mask & 15))))
        stage_mode = 1;
    else if (splits == 1 && Cf && !Cb && !mask && bn <= 112 && ldc % 4 == 0 &&
             !((uintptr_t)Cf & 15))
        stage_mode = 2;
    const int vec_atomic = splits > 1 && ldc % 4 == 0 && !((uintptr_t)Cf & 15);
    if (attr_err != cudaSuccess) return PCAGB_ECUDA;
    dim3 grid((N + bn - 1) / bn, (M + kGRows - 1) / kGRows, splits);
    k_gemm_tc<<<grid, 128, smem, (cudaStream_t)stream>>>(
        ma, mb, bias, (const __nv_bfloat16 *)mask, ldm, (__nv_bfloat16 *)Cb, Cf, ldc, M, N,
        kblocks, per, bn, idesc, tcols, relu, splits > 1, stage_mode, vec_atomic, 0, status);
    return cudaGetLastError() == cudaSuccess ? PCAGB_OK : PCAGB_ECUDA;
}

/* Tensor map of a [krows][cols] bf16 matrix (row stride ld elements) read
   as an MN-major operand: boxes of 64 columns x 64 rows, 128-byte swizzle. */
bool tile_map_mn(CUtensorMap *m, const void *ptr, int krows, int cols, int ld)
{
    EncodeTiledFn fn = encode_fn();
    if (!fn) return false;
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)krows};
    cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    cuuint32_t box[2] = {64, 64};
    cuuint32_t estr[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(ptr), dims, strides, box,
              estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
              CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

/* C[i] += the `splits` slabs' values at i, in slab order. */
__global__ void k_split_sum(const float *part, int splits, size_t count, float *C)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += (size_t)gridDim.x * blockDim.x) {
        float v = 0.f;
        for (int z = 0; z < splits; z++) v += part[(size_t)z * count + i];
        C[i] += v;
    }
}

/* The number of K splits pcagb_vnet_wgrad_tc uses for this shape when asked
 * for `splits` (its partial buffer holds that many [M][ldc] slabs). */
extern "C" int pcagb_vnet_wgrad_splits(int K, int splits)
{
    const int kblocks = (K + kGBK - 1) / kGBK;
    if (splits < 1) splits = 1;
    if (splits > kblocks) splits = kblocks;
    const int per = (kblocks + splits - 1) / splits;
    return (kblocks + per - 1) / per;
}

/* Weight gradient on tcgen05 without transposes: C[M][N] += dY^T . X over
 * K rows, dY [K][M] (leading dimension ldy) and X [K][N] (ldx) read as
 * stored (MN-major operands), with the K rows in `splits` ranges. With
 * `part` (pcagb_vnet_wgrad_splits(K, splits) slabs of M x ldc floats) each
 * range writes its own slab and the slabs are added into C in range order,
 * so the result is the same on every run; without it the ranges' fp32 sums
 * are added into C atomically. C is zeroed by the caller (leading dimension
 * ldc). ldy and ldx are multiples of 8 elements, dY and X 16-byte aligned. */
extern "C" int pcagb_vnet_wgrad_tc(const void *dY, int ldy, const void *X, int ldx, float *C,
                                   int ldc, int M, int N, int K, int splits, float *part,
                                   int *status, void *stream)
{
    if (M <= 0 || N <= 0 || K <= 0) return PCAGB_OK;
    if (!dY || !X || !C || !status || (ldy & 7) || (ldx & 7) || ldy < M || ldx < N ||
        ldc < N || ((uintptr_t)dY & 15) || ((uintptr_t)X & 15) || splits < 1)
        return PCAGB_EINVAL;
    const int bn = N > 192 ? 256 : (N + 63) / 64 * 64;
    uint32_t tcols = 32;
    while (tcols < (uint32_t)bn) tcols <<= 1;
    CUtensorMap ma, mb;
    if (!tile_map_mn(&ma, dY, K, M, ldy) || !tile_map_mn(&mb, X, K, N, ldx)) return PCAGB_ECUDA;
    const int kblocks = (K + kGBK - 1) / kGBK;
    if (splits > kblocks) splits = kblocks;
    const int per = (kblocks + splits - 1) / splits;
    splits = (kblocks + per - 1) / per;
    /* bits 15 and 16: A and B MN-major */
    const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | (1u << 15) | (1u << 16) |
                           ((uint32_t)(bn >> 3) << 17) | ((uint32_t)(kGRows >> 4) << 24);
    const int smem = kGStages * (kGABytes + bn * 128) + 256 + 1024 + 1024;
    static std::once_flag attr_once;
    static cudaError_t attr_err = cudaSuccess;
    std::call_once(attr_once, [] {
        attr_err = cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        kGStages * (kGABytes + 256 * 128) + 256 + 2048);
    });
    if (attr_err != cudaSuccess) return PCAGB_ECUDA;
    float *out = part ? part : C;
    const int vec_atomic = ldc % 4 == 0 && !((uintptr_t)out & 15);
    dim3 grid((N + bn - 1) / bn, (M + kGRows - 1) / kGRows, splits);
    k_gemm_tc<<<grid, 128, smem, (cudaStream_t)stream>>>(
        ma, mb, nullptr, nullptr, 0, nullptr, out, ldc, M, N, kblocks, per, bn, idesc, tcols, 0,
        part ? 2 : 1, 0, vec_atomic, 1, status);
    if (cudaGetLastError() != cudaSuccess) return PCAGB_ECUDA;
    if (part) {
        const size_t count = (size_t)M * ldc;
        const unsigned blocks = (unsigned)std::min<size_t>((count + 255) / 256, 4096);
        k_split_sum<<<blocks, 256, 0, (cudaStream_t)stream>>>(part, splits, count, C);
        if (cudaGetLastError() != cudaSuccess) return PCAGB_ECUDA;
    }
    return PCAGB_OK;
}


extern "C" int pcagb_vnet_encode_pool_tc(const void *W1, const float *b1, const void *W2,
                                         const float *b2, const uint16_t *regs,
                                         const uint8_t *flags, const uint8_t *live,
                                         const uint16_t *task, const uint8_t *depth, int TP, int n,
                                         const uint16_t *task_io, const int32_t *task_T, void *P,
                                         int *status, void *stream)
{
    if (n <= 0) return PCAGB_OK;
    if ((TP != 16 && TP != 32) || !W1 || !W2 || !b1 || !b2 || !P || !status ||
        ((uintptr_t)W1 & 15) || ((uintptr_t)W2 & 15))
        return PCAGB_EINVAL;
    CUtensorMap m1, m2;
    if (!weight_map(&m1, W1, kFeat) || !weight_map(&m2, W2, kUnits)) return PCAGB_ECUDA;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return PCAGB_ECUDA;
    static std::once_flag attr_once;
    static cudaError_t attr_err = cudaSuccess;
    std::call_once(attr_once, [] {
        attr_err = cudaFuncSetAttribute(k_encode_pool_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        kSmemBytes);
    });
    if (attr_err != cudaSuccess) return PCAGB_ECUDA;
    const int ntiles = (n + kStatesPerTile - 1) / kStatesPerTile;
    const int grid = ntiles < sms ? ntiles : sms;
    k_encode_pool_tc<<<grid, kThreads, kSmemBytes, (cudaStream_t)stream>>>(
        m1, m2, b1, b2, regs, flags, live, task, depth, TP, n, task_io, task_T,
        (__nv_bfloat16 *)P, status);
    return cudaGetLastError() == cudaSuccess ? PCAGB_OK : PCAGB_ECUDA;
}
