/*
 * pca_isa.h -- PCA-16 branchless semantics shared by the host library and
 * the CUDA kernels.
 *
 * Encoding (src/pca.h:91-102 of the reference):
 *   R type [op:5][rd:3][rs:3][rt:3][pad:2], I type [op:5][rd:3][imm:8].
 * Branchless step semantics follow src/search_state.c:49-187: ADD/SUB/ADDI
 * set ZNCV, MUL sets ZNC, logic and shifts set ZN, LDI leaves the flags,
 * shift amounts are masked to 4 bits, r0 reads as zero.
 *
 * Kernels never decode raw instructions in their inner loops. Every
 * candidate is pre-decoded on the host into a 32-bit "micro-op":
 *   bits 0-4 op, 5-7 rd, 8-10 a-operand register, 11-13 b-operand register,
 *   16-23 imm8.
 * ADDI reads its destination, so its a-operand register is rd; LDI reads no
 * register. With that, every op is res = f(op, R[a], R[b], imm).
 */
#ifndef PCA_ISA_H
#define PCA_ISA_H

#include <stdint.h>

#if defined(__CUDACC__)
#define PCA_HD __host__ __device__ __forceinline__
#else
#define PCA_HD static inline
#endif

enum {
    PCA_OP_NOP = 0x00, PCA_OP_HLT = 0x01, PCA_OP_ADD = 0x02, PCA_OP_SUB = 0x03,
    PCA_OP_MUL = 0x04, PCA_OP_DIV = 0x05, PCA_OP_MOD = 0x06, PCA_OP_AND = 0x07,
    PCA_OP_OR = 0x08, PCA_OP_XOR = 0x09, PCA_OP_SHL = 0x0A, PCA_OP_SHR = 0x0B,
    PCA_OP_ASR = 0x0C, PCA_OP_CMP = 0x0D, PCA_OP_LD = 0x0E, PCA_OP_ST = 0x0F,
    PCA_OP_LDI = 0x10, PCA_OP_LUI = 0x11, PCA_OP_ADDI = 0x12, PCA_OP_BR = 0x13,
    PCA_OP_JMP = 0x14, PCA_OP_CALL = 0x15, PCA_OP_RET = 0x16, PCA_OP_IN = 0x17,
    PCA_OP_OUT = 0x18
};

#define PCA_FZ 0x01u
#define PCA_FN 0x02u
#define PCA_FC 0x04u
#define PCA_FV 0x08u

#define PCA_INSN_OP(i)  (((i) >> 11) & 0x1Fu)
#define PCA_INSN_RD(i)  (((i) >> 8) & 7u)
#define PCA_INSN_RS(i)  (((i) >> 5) & 7u)
#define PCA_INSN_RT(i)  (((i) >> 2) & 7u)
#define PCA_INSN_IMM(i) ((i) & 0xFFu)
#define PCA_ENC_R(op, rd, rs, rt) \
    ((uint16_t)((((op) & 0x1Fu) << 11) | (((rd) & 7u) << 8) | (((rs) & 7u) << 5) | (((rt) & 7u) << 2)))
#define PCA_ENC_I(op, rd, imm) \
    ((uint16_t)((((op) & 0x1Fu) << 11) | (((rd) & 7u) << 8) | ((imm) & 0xFFu)))

/* micro-op fields */
#define UOP_OP(u)  ((u) & 0x1Fu)
#define UOP_RD(u)  (((u) >> 5) & 7u)
#define UOP_A(u)   (((u) >> 8) & 7u)
#define UOP_B(u)   (((u) >> 11) & 7u)
#define UOP_IMM(u) (((u) >> 16) & 0xFFu)

PCA_HD uint32_t pca_uop_from_insn(uint32_t insn)
{
    uint32_t op = PCA_INSN_OP(insn), rd = PCA_INSN_RD(insn);
    uint32_t a = PCA_INSN_RS(insn), b = PCA_INSN_RT(insn), imm = PCA_INSN_IMM(insn);
    if (op == PCA_OP_ADDI) { a = rd; b = 0; }
    if (op == PCA_OP_LDI) { a = 0; b = 0; }
    if (op == PCA_OP_ADDI || op == PCA_OP_LDI) return op | (rd << 5) | (a << 8) | (b << 11) | (imm << 16);
    return op | (rd << 5) | (a << 8) | (b << 11);
}

/* The value an op writes into rd, for one test (16-bit result in 32 bits). */
PCA_HD uint32_t pca_alu(uint32_t op, uint32_t a, uint32_t b, uint32_t imm)
{
    switch (op) {
    case PCA_OP_ADD: return (a + b) & 0xFFFFu;
    case PCA_OP_SUB: return (a - b) & 0xFFFFu;
    case PCA_OP_MUL: return (a * b) & 0xFFFFu;
    case PCA_OP_AND: return a & b;
    case PCA_OP_OR:  return a | b;
    case PCA_OP_XOR: return a ^ b;
    case PCA_OP_SHL: return (a << (b & 15u)) & 0xFFFFu;
    case PCA_OP_SHR: return a >> (b & 15u);
    case PCA_OP_ASR: return (uint32_t)(uint16_t)((int16_t)(uint16_t)a >> (b & 15u));
    case PCA_OP_LDI: return imm;
    case PCA_OP_ADDI: return (a + (uint32_t)(int32_t)(int8_t)(uint8_t)imm) & 0xFFFFu;
    default: return 0x10000u; /* never equals a 16-bit value */
    }
}

PCA_HD uint32_t pca_zn(uint32_t r)
{
    return (r == 0 ? PCA_FZ : 0u) | ((r & 0x8000u) ? PCA_FN : 0u);
}

/* Flags after an op (src/search_state.c:80-176); LDI keeps old_flags. */
PCA_HD uint32_t pca_alu_flags(uint32_t op, uint32_t a, uint32_t b, uint32_t imm,
                              uint32_t res, uint32_t old_flags)
{
    switch (op) {
    case PCA_OP_ADD:
        return pca_zn(res) | ((a + b) > 0xFFFFu ? PCA_FC : 0u) |
               ((~(a ^ b) & (a ^ res) & 0x8000u) ? PCA_FV : 0u);
    case PCA_OP_SUB:
        return pca_zn(res) | (a >= b ? PCA_FC : 0u) |
               (((a ^ b) & (a ^ res) & 0x8000u) ? PCA_FV : 0u);
    case PCA_OP_MUL:
        return pca_zn(res) | ((a * b) > 0xFFFFu ? PCA_FC : 0u);
    case PCA_OP_LDI:
        return old_flags;
    case PCA_OP_ADDI: {
        uint32_t e = (uint32_t)(uint16_t)(int16_t)(int8_t)(uint8_t)imm;
        return pca_zn(res) | ((a + e) > 0xFFFFu ? PCA_FC : 0u) |
               ((~(a ^ e) & (a ^ res) & 0x8000u) ? PCA_FV : 0u);
    }
    default:
        return pca_zn(res);
    }
}

#endif
