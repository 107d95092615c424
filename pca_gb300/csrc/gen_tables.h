/*
 * gen_tables.h -- the branchless candidate generator, precomputed for all
 * 128 liveness masks.
 *
 * The generator is the reference's src/search_state.c:280-330: nine ALU ops
 * (ADD SUB MUL AND OR XOR SHL SHR ASR) over rd = r1..r7 and live source
 * registers (r0 always allowed), with rt >= rs for the commutative ops and
 * five no-op encodings skipped; then LDI rd, {0,1,2,3,4,5,8,16,32,64,128,255}
 * for every rd; then ADDI rd, {-1,1,-2,2,-3,3} for live rd. The list order is
 * the reference's DFS order, which the engine preserves.
 *
 * A liveness mask only matters in bits 1..7, so masks are indexed by
 * live >> 1 (0..127).
 *
 * Value classes. The value an instruction writes does not depend on its
 * destination register unless the op reads it (ADDI). At the last kernel
 * position only that value matters, so candidates that differ only in rd
 * form one value class, evaluated once: (op, a, b, imm) with rd cleared, or
 * with rd kept for ADDI.
 */
#ifndef PCA_GEN_TABLES_H
#define PCA_GEN_TABLES_H

#include <stdint.h>
#include <vector>

#include "pca_isa.h"

namespace pcagb {

struct GenTables {
    /* per mask (128): offsets into the flat arrays, size 129 */
    std::vector<uint32_t> cand_off;
    std::vector<uint16_t> cand;        /* raw instruction words            */
    std::vector<uint32_t> cand_uop;    /* pre-decoded micro-ops            */
    std::vector<uint16_t> cand_vc;     /* value class index within mask    */
    std::vector<uint32_t> vc_off;      /* size 129                         */
    std::vector<uint32_t> vc_uop;      /* one micro-op per value class     */
    /* per mask: runs of <= 32 consecutive candidates with one op, so a warp
       expanding a state works on a single op at a time; entry =
       start << 8 | count, start relative to the mask's candidate list */
    std::vector<uint32_t> chunk_off;   /* size 129 */
    std::vector<uint32_t> chunks;
    /* f[s][m]: programs decided by s more instructions from mask m:
       f[1][m] = nc(m), f[s][m] = sum over candidates c of f[s-1][m | rd(c)] */
    std::vector<uint64_t> f[5];
    /* ev[s][m]: value-class evaluations of a suffix of s instructions from
       mask m: ev[1][m] = nvc(m), ev[s][m] = sum over candidates c of
       ev[s-1][m | rd(c)] (the suffix kernels' unit of work) */
    std::vector<uint64_t> ev[5];
    /* the value classes of mask m that read register r (1..7): class
       indices (within the mask's list) vcr[vcr_off[m*8+r] .. vcr_off[m*8+r+1]) */
    std::vector<uint32_t> vcr_off;     /* size 128*8+1 */
    std::vector<uint16_t> vcr;
    /* The same classes grouped by operand pair, for evaluating every op of
       a pair at once: entry = a | b << 3 | opmask << 6 | imm << 16, where
       opmask bit k < 9 is the ALU op kPairOps[k] on (a, b) and bit 9 an ADDI
       on register a with immediate imm (an ADDI class per entry).
       pr_cls[entry * 10 + k] = that class's index in the mask's list. */
    /* cand_dupe[i]: candidate i writes the same value and flags as an
       earlier candidate of its mask on every state (copies of one register
       with its Z/N flags, zero with Z, zero with Z and C); a child by it is
       that sibling's state and never its representative */
    std::vector<uint8_t> cand_dupe;
    std::vector<uint32_t> pr_off;      /* size 128*8+1 */
    std::vector<uint32_t> pr;
    std::vector<uint16_t> pr_cls;
    /* pr_ev[m*8+r]: class evaluations one pass over the pair list of (m, r)
       runs (every admitted op of every entry) */
    std::vector<uint32_t> pr_ev;
    int max_nc = 0;
    int max_nvc = 0;

    int nc(int mask) const { return (int)(cand_off[mask + 1] - cand_off[mask]); }
    int nvc(int mask) const { return (int)(vc_off[mask + 1] - vc_off[mask]); }
};

/* Upper bound on the candidates of all 128 masks together (130,144 with the
   current generator): fixed-size device tables are sized by it, and a CPU
   test checks the generator stays within it. */
constexpr uint32_t kMaxTableCandidates = 131072;

/* The ALU ops of an operand-pair entry, by opmask bit. */
static const uint32_t kPairOps[9] = {PCA_OP_ADD, PCA_OP_SUB, PCA_OP_MUL, PCA_OP_AND, PCA_OP_OR,
                                     PCA_OP_XOR, PCA_OP_SHL, PCA_OP_SHR, PCA_OP_ASR};

/* Built once (thread-safe, immutable afterwards). */
const GenTables &gen_tables();

/* The generator for one live mask, in reference order. */
int gen_candidates(uint8_t live, uint16_t *out, int max);

}  // namespace pcagb

#endif
