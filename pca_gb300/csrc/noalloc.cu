/*
 * noalloc.cu -- pcagb_solve_small_noalloc: a solve that allocates nothing.
 *
 * Some callers cannot call cudaMalloc: a host process whose device memory is
 * owned by another allocator (a framework's caching pool that has reserved
 * the free HBM, so a raw cudaMalloc fails or fragments it), code that must not
 * take the implicit device synchronisation cudaMalloc/cudaFree can cause in
 * the middle of latency-critical work, and plugin hosts that forbid a
 * library from owning device memory at all. pcagb_solve and pcagb_complete
 * need an engine (pcagb_engine_create allocates an HBM arena); this entry
 * point does not.
 *
 * It runs the suffix kernel straight from the task root (no OEP levels), so
 * it enumerates every kernel program of length K = 1..3 and returns the full
 * canonical program set at the optimal length, like pcagb_solve with
 * split_depth 0. Its scratch -- the root state, the solution counters and the
 * solving records -- lives in g_noalloc_scratch, a file-scope static
 * __device__ array of PCAGB_NOALLOC_SCRATCH_BYTES (16 MiB): every GPU that
 * loads this library holds it until the process exits. The candidate tables
 * live in fixed static __device__ arrays as well.
 *
 * Set-up: the first call on a device (with that device current) resolves the
 * scratch's device address with cudaGetSymbolAddress and uploads the
 * candidate tables with cudaMemcpyToSymbol, and loads all three suffix
 * kernels (CUDA would otherwise load each at its first launch, taking device
 * memory then); later calls on that device reuse them. Make the first call
 * on each device before any stream capture.
 *
 * Every call shares the one scratch array, which keeps the last call's
 * contents; each call clears the counters it needs before its kernels run.
 * Calls whose work overlaps on the GPU (other host threads, or other streams
 * without ordering between them) race on the scratch: serialise them.
 */
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/pca_gb300.h"
#include "gen_tables.h"
#include "pca_isa.h"

namespace {

constexpr uint32_t kNaMaxCand = pcagb::kMaxTableCandidates;
constexpr uint64_t kNaHeader = 4096;      /* counters + root state        */
constexpr uint64_t kNaMaxRecords =
    (PCAGB_NOALLOC_SCRATCH_BYTES - kNaHeader) / sizeof(ulonglong2);

/* The scratch: [0] solving-record count, [8] overflow flag, [256..] root
 * state (regs u16[8][32], flags u8[32], live), [4096..] records. */
static __device__ __align__(256) unsigned char g_noalloc_scratch[PCAGB_NOALLOC_SCRATCH_BYTES];

/* Candidate tables of the generator (src/search_state.c:280-330). */
static __device__ __align__(256) uint32_t g_na_cand_uop[kNaMaxCand];
static __device__ __align__(256) uint32_t g_na_vc_uop[kNaMaxCand];
static __constant__ uint32_t c_na_cand_off[129];
static __constant__ uint32_t c_na_vc_off[129];

struct NaPtrs {
    unsigned char *scratch;
    const uint32_t *cand_uop;
    const uint32_t *vc_uop;
};

struct NaTask {
    int T;
    uint32_t target[32];
};

constexpr int kNaWarps = 8;

/* Columns r0..r7 of the root, two spare columns for the middle
 * instructions, one word of padding per row. */
struct NaState {
    uint32_t R[10][33];
};

__device__ __forceinline__ void na_record(const NaPtrs &P, uint32_t m1, uint32_t m2, uint32_t vc)
{
    unsigned long long *count = (unsigned long long *)P.scratch;
    unsigned long long slot = atomicAdd(count, 1ull);
    if (slot < kNaMaxRecords) {
        ulonglong2 *rec = (ulonglong2 *)(P.scratch + kNaHeader);
        rec[slot] = make_ulonglong2(0, ((unsigned long long)m1 << 32) | (m2 << 16) | vc);
    } else {
        ((unsigned int *)P.scratch)[2] = 1u;
    }
}

/* Value classes of mask m against the warp's state (test 0 first, then all
 * tests at once for the survivors); rd1/rd2 remap to spare columns 8/9. */
__device__ void na_scan(const NaPtrs &P, const NaState &S, const NaTask &task, uint32_t m,
                        uint32_t rd1, uint32_t rd2, uint32_t tgt, int lane, uint32_t m1,
                        uint32_t m2)
{
    const uint32_t vb = c_na_vc_off[m], nvc = c_na_vc_off[m + 1] - vb;
    for (uint32_t b0 = 0; b0 < nvc; b0 += 32) {
        const uint32_t i = b0 + lane;
        uint32_t u = 0;
        bool pass = false;
        if (i < nvc) {
            u = P.vc_uop[vb + i];
            uint32_t ra = UOP_A(u), rb = UOP_B(u);
            ra = ra == rd2 ? 9u : ra == rd1 ? 8u : ra;
            rb = rb == rd2 ? 9u : rb == rd1 ? 8u : rb;
            pass = pca_alu(UOP_OP(u), S.R[ra][0], S.R[rb][0], UOP_IMM(u)) == task.target[0];
        }
        uint32_t bal = __ballot_sync(0xFFFFFFFFu, pass);
        while (bal) {
            const int j = __ffs(bal) - 1;
            bal &= bal - 1;
            const uint32_t uj = __shfl_sync(0xFFFFFFFFu, u, j);
            uint32_t ra = UOP_A(uj), rb = UOP_B(uj);
            ra = ra == rd2 ? 9u : ra == rd1 ? 8u : ra;
            rb = rb == rd2 ? 9u : rb == rd1 ? 8u : rb;
            bool ok = lane >= task.T ||
                      pca_alu(UOP_OP(uj), S.R[ra][lane], S.R[rb][lane], UOP_IMM(uj)) == tgt;
            if (__all_sync(0xFFFFFFFFu, ok) && lane == 0) na_record(P, m1, m2, b0 + j);
        }
    }
}

/* Suffix enumeration of depth SD from the root held in the scratch. Work
 * item = first instruction (SD >= 2) or the whole root (SD == 1). */
template <int SD>
__global__ void __launch_bounds__(kNaWarps * 32) k_suffix_noalloc(NaPtrs P, NaTask task)
{
    __shared__ NaState sst[kNaWarps];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    NaState &S = sst[w];
    const uint16_t *root = (const uint16_t *)(P.scratch + 256);
    const uint32_t live = P.scratch[256 + 8 * 32 * 2 + 32];
    for (int r = 0; r < 8; r++) S.R[r][lane] = lane < task.T ? root[r * 32 + lane] : 0u;
    __syncwarp();
    const uint32_t tgt = lane < task.T ? task.target[lane] : 0u;
    const uint32_t m0 = (live >> 1) & 127u;
    const uint32_t cb0 = c_na_cand_off[m0], nc0 = c_na_cand_off[m0 + 1] - cb0;
    const uint32_t items = SD == 1 ? 1u : nc0;
    for (uint32_t it = blockIdx.x * kNaWarps + w; it < items; it += gridDim.x * kNaWarps) {
        if (SD == 1) {
            na_scan(P, S, task, m0, 8, 8, tgt, lane, 0, 0);
            continue;
        }
        const uint32_t u1 = P.cand_uop[cb0 + it], rd1 = UOP_RD(u1);
        __syncwarp();
        S.R[8][lane] = lane < task.T ? pca_alu(UOP_OP(u1), S.R[UOP_A(u1)][lane],
                                               S.R[UOP_B(u1)][lane], UOP_IMM(u1))
                                     : 0u;
        __syncwarp();
        const uint32_t m1 = (m0 | (1u << (rd1 - 1))) & 127u;
        if (SD == 2) {
            na_scan(P, S, task, m1, rd1, 8, tgt, lane, it, 0);
            continue;
        }
        const uint32_t cb1 = c_na_cand_off[m1], nc1 = c_na_cand_off[m1 + 1] - cb1;
        for (uint32_t i2 = 0; i2 < nc1; i2++) {
            const uint32_t u2 = P.cand_uop[cb1 + i2], rd2 = UOP_RD(u2);
            uint32_t ra = UOP_A(u2), rb = UOP_B(u2);
            ra = ra == rd1 ? 8u : ra;
            rb = rb == rd1 ? 8u : rb;
            __syncwarp();
            S.R[9][lane] = lane < task.T ? pca_alu(UOP_OP(u2), S.R[ra][lane], S.R[rb][lane],
                                                   UOP_IMM(u2))
                                         : 0u;
            __syncwarp();
            const uint32_t m2 = (m1 | (1u << (rd2 - 1))) & 127u;
            na_scan(P, S, task, m2, rd2 == rd1 ? 8u : rd1, rd2, tgt, lane, it, i2);
        }
    }
}

thread_local char t_na_err[256];

void na_set_err(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(t_na_err, sizeof t_na_err, fmt, ap);
    va_end(ap);
}

/* Per-device set-up: scratch address and candidate tables. */
std::mutex g_na_mu;
NaPtrs g_na_ptrs[64];
bool g_na_ready[64];

int na_setup(int dev, NaPtrs *out)
{
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (dev < 0 || dev >= 64) { na_set_err("device %d out of range", dev); return PCAGB_EINVAL; }
    if (g_na_ready[dev]) { *out = g_na_ptrs[dev]; return PCAGB_OK; }
    const pcagb::GenTables &gt = pcagb::gen_tables();
    if (gt.cand_uop.size() > kNaMaxCand || gt.vc_uop.size() > kNaMaxCand) {
        na_set_err("candidate tables exceed the static arrays");
        return PCAGB_ELIMIT;
    }
    NaPtrs p{};
    cudaError_t err = cudaGetSymbolAddress((void **)&p.scratch, g_noalloc_scratch);
    if (err == cudaSuccess) err = cudaGetSymbolAddress((void **)&p.cand_uop, g_na_cand_uop);
    if (err == cudaSuccess) err = cudaGetSymbolAddress((void **)&p.vc_uop, g_na_vc_uop);
    if (err == cudaSuccess)
        err = cudaMemcpyToSymbol(g_na_cand_uop, gt.cand_uop.data(), gt.cand_uop.size() * 4);
    if (err == cudaSuccess)
        err = cudaMemcpyToSymbol(g_na_vc_uop, gt.vc_uop.data(), gt.vc_uop.size() * 4);
    if (err == cudaSuccess) err = cudaMemcpyToSymbol(c_na_cand_off, gt.cand_off.data(), 129 * 4);
    if (err == cudaSuccess) err = cudaMemcpyToSymbol(c_na_vc_off, gt.vc_off.data(), 129 * 4);
    /* CUDA loads a kernel lazily, at its first launch, and loading takes
       device memory. Load all three suffix depths here, so that a later call
       that first reaches a deeper kernel allocates nothing. */
    cudaFuncAttributes fa;
    if (err == cudaSuccess) err = cudaFuncGetAttributes(&fa, k_suffix_noalloc<1>);
    if (err == cudaSuccess) err = cudaFuncGetAttributes(&fa, k_suffix_noalloc<2>);
    if (err == cudaSuccess) err = cudaFuncGetAttributes(&fa, k_suffix_noalloc<3>);
    if (err != cudaSuccess) {
        na_set_err("no-allocation set-up on device %d failed: %s", dev, cudaGetErrorString(err));
        return PCAGB_ECUDA;
    }
    g_na_ptrs[dev] = p;
    g_na_ready[dev] = true;
    *out = p;
    return PCAGB_OK;
}

}  // namespace

extern "C" {

const char *pcagb_noalloc_last_error(void) { return t_na_err; }

int pcagb_solve_small_noalloc(const task_spec_t *task, int max_depth, void *stream,
                              int *optimal_depth, uint64_t *total_solutions,
                              uint16_t *sol_progs, int *sol_lens, int sol_cap)
{
    t_na_err[0] = 0;
    if (!task || !optimal_depth || !total_solutions) {
        na_set_err("null argument");
        return PCAGB_EINVAL;
    }
    *optimal_depth = -1;
    *total_solutions = 0;
    if (max_depth < 0 || max_depth > PCAGB_NOALLOC_MAX_DEPTH) {
        na_set_err("max_depth %d is beyond the no-allocation limit of %d instructions", max_depth,
                   PCAGB_NOALLOC_MAX_DEPTH);
        return PCAGB_EINVAL;
    }
    if (task->num_outputs != 1 || task->num_tests < 1 || task->num_tests > MAX_TESTS ||
        task->num_inputs < 0 || task->num_inputs > 7) {
        na_set_err("task needs 1..32 tests, one output and at most 7 inputs");
        return PCAGB_EINVAL;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        na_set_err("no CUDA device: the PCA-16 engine runs only on the GPU");
        return PCAGB_ENODEV;
    }
    NaPtrs P;
    int rc = na_setup(dev, &P);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;

    /* root state into the scratch (regs u16[8][32], flags, live) */
    unsigned char root[8 * 32 * 2 + 32 + 8];
    memset(root, 0, sizeof root);
    uint16_t *regs = (uint16_t *)root;
    uint8_t live = 0;
    for (int i = 0; i < task->num_inputs; i++) {
        live |= (uint8_t)(1u << (i + 1));
        for (int t = 0; t < task->num_tests; t++) regs[(i + 1) * 32 + t] = task->tests[t].in[i];
    }
    root[8 * 32 * 2 + 32] = live;
    NaTask td{};
    td.T = task->num_tests;
    for (int t = 0; t < td.T; t++) td.target[t] = task->tests[t].out[0];

    const pcagb::GenTables &gt = pcagb::gen_tables();
    int stored = 0;
    auto emit = [&](const uint16_t *kernel, int klen, uint32_t out_reg) {
        if (stored < sol_cap && sol_progs) {
            uint16_t *p = sol_progs + (size_t)stored * 16;
            memset(p, 0, 32);
            int n = 0;
            for (int i = 0; i < task->num_inputs; i++)
                p[n++] = PCA_ENC_I(PCA_OP_IN, i + 1, task->input_ports[i]);
            for (int i = 0; i < klen; i++) p[n++] = kernel[i];
            p[n++] = PCA_ENC_I(PCA_OP_OUT, out_reg, task->output_ports[0]);
            p[n++] = PCA_ENC_R(PCA_OP_HLT, 0, 0, 0);
            if (sol_lens) sol_lens[stored] = n;
            stored++;
        }
        (*total_solutions)++;
    };

    /* K = 0: a live input register already holds the target */
    for (uint32_t r = 1; r < 8; r++) {
        if (!((live >> r) & 1u)) continue;
        bool ok = true;
        for (int t = 0; t < td.T && ok; t++) ok = task->tests[t].in[r - 1] == task->tests[t].out[0];
        if (ok) emit(nullptr, 0, r);
    }
    if (*total_solutions) {
        *optimal_depth = 0;
        return 1;
    }
    cudaError_t err = cudaMemcpyAsync(P.scratch + 256, root, sizeof root, cudaMemcpyHostToDevice, st);
    for (int K = 1; K <= max_depth && err == cudaSuccess; K++) {
        err = cudaMemsetAsync(P.scratch, 0, 16, st);  /* count + overflow flag */
        if (err != cudaSuccess) break;
        if (K == 1) k_suffix_noalloc<1><<<1, kNaWarps * 32, 0, st>>>(P, td);
        else if (K == 2) k_suffix_noalloc<2><<<16, kNaWarps * 32, 0, st>>>(P, td);
        else k_suffix_noalloc<3><<<256, kNaWarps * 32, 0, st>>>(P, td);
        err = cudaGetLastError();
        unsigned long long hdr[2] = {0, 0};
        if (err == cudaSuccess) err = cudaMemcpyAsync(hdr, P.scratch, 16, cudaMemcpyDeviceToHost, st);
        if (err == cudaSuccess) err = cudaStreamSynchronize(st);
        if (err != cudaSuccess) break;
        const uint64_t nrec = hdr[0];
        if (hdr[1] & 1u) {
            na_set_err("%llu solving records exceed the %llu the scratch holds",
                       (unsigned long long)nrec, (unsigned long long)kNaMaxRecords);
            return PCAGB_ELIMIT;
        }
        if (!nrec) continue;
        *optimal_depth = K;
        /* decode records in chunks through a stack buffer */
        const uint32_t m_root = (live >> 1) & 127u;
        ulonglong2 chunk[256];
        for (uint64_t base = 0; base < nrec && err == cudaSuccess; base += 256) {
            const uint64_t n = nrec - base < 256 ? nrec - base : 256;
            err = cudaMemcpyAsync(chunk, P.scratch + kNaHeader + base * sizeof(ulonglong2),
                                  n * sizeof(ulonglong2), cudaMemcpyDeviceToHost, st);
            if (err == cudaSuccess) err = cudaStreamSynchronize(st);
            for (uint64_t i = 0; i < n && err == cudaSuccess; i++) {
                const uint32_t c1 = (uint32_t)(chunk[i].y >> 32);
                const uint32_t c2 = (uint32_t)((chunk[i].y >> 16) & 0xFFFF);
                const uint32_t vc = (uint32_t)(chunk[i].y & 0xFFFF);
                uint16_t kernel[3];
                int klen = 0;
                uint32_t m = m_root;
                auto take = [&](uint32_t c) {
                    const uint32_t idx = gt.cand_off[m] + c;
                    kernel[klen++] = gt.cand[idx];
                    m |= 1u << (UOP_RD(gt.cand_uop[idx]) - 1);
                };
                if (K >= 2) take(c1);
                if (K >= 3) take(c2);
                for (uint32_t c = 0; c < (uint32_t)gt.nc(m); c++) {
                    const uint32_t idx = gt.cand_off[m] + c;
                    if (gt.cand_vc[idx] != vc) continue;
                    kernel[klen] = gt.cand[idx];
                    emit(kernel, klen + 1, UOP_RD(gt.cand_uop[idx]));
                }
            }
        }
        break;
    }
    if (err != cudaSuccess) {
        na_set_err("CUDA error in the no-allocation solve: %s", cudaGetErrorString(err));
        return PCAGB_ECUDA;
    }
    return *optimal_depth >= 0 ? 1 : 0;
}

}  // extern "C"
