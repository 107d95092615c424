/*
 * pca_oracle.c -- CPU restatement of the reference PCA-16 branchless search.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the checker for the GPU engine: the
 * tests, the smoke check and bench.py's CPU-baseline leg call it; the product
 * library never links it. Each function cites the reference file:line whose
 * behaviour it restates. Plain C99 + POSIX threads.
 */
#define _POSIX_C_SOURCE 199309L
#include "pca_oracle.h"

#include <ctype.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* ---- ISA constants (src/pca.h:32-102) ---------------------------------- */
enum {
    OP_NOP = 0x00, OP_HLT = 0x01, OP_ADD = 0x02, OP_SUB = 0x03, OP_MUL = 0x04,
    OP_DIV = 0x05, OP_MOD = 0x06, OP_AND = 0x07, OP_OR = 0x08, OP_XOR = 0x09,
    OP_SHL = 0x0A, OP_SHR = 0x0B, OP_ASR = 0x0C, OP_CMP = 0x0D, OP_LD = 0x0E,
    OP_ST = 0x0F, OP_LDI = 0x10, OP_LUI = 0x11, OP_ADDI = 0x12, OP_BR = 0x13,
    OP_JMP = 0x14, OP_CALL = 0x15, OP_RET = 0x16, OP_IN = 0x17, OP_OUT = 0x18
};
#define F_Z 0x01
#define F_N 0x02
#define F_C 0x04
#define F_V 0x08
#define I_OP(i)   (((i) >> 11) & 0x1F)
#define I_RD(i)   (((i) >> 8) & 7)
#define I_RS(i)   (((i) >> 5) & 7)
#define I_RT(i)   (((i) >> 2) & 7)
#define I_IMM(i)  ((i) & 0xFF)
#define ENC_R(op, rd, rs, rt) \
    ((uint16_t)(((op) & 0x1F) << 11 | ((rd) & 7) << 8 | ((rs) & 7) << 5 | ((rt) & 7) << 2))
#define ENC_I(op, rd, imm) \
    ((uint16_t)(((op) & 0x1F) << 11 | ((rd) & 7) << 8 | ((imm) & 0xFF)))

/* ---- task JSON loader (tasks/spec.c:15-184) ----------------------------- */

static const char *skip_ws(const char *p)
{
    while (*p && isspace((unsigned char)*p)) p++;
    return p;
}

static const char *find_key(const char *json, const char *key)
{
    char pat[128];
    snprintf(pat, sizeof pat, "\"%s\"", key);
    const char *p = strstr(json, pat);
    if (!p) return NULL;
    p = skip_ws(p + strlen(pat));
    if (*p == ':') p++;
    return skip_ws(p);
}

static const char *parse_ints(const char *p, long *arr, int maxlen, int *count)
{
    p = skip_ws(p);
    *count = 0;
    if (*p != '[') return NULL;
    p++;
    while (*count < maxlen) {
        p = skip_ws(p);
        if (*p == ']') return p + 1;
        if (*p == ',') p++;
        char *end;
        arr[*count] = strtol(skip_ws(p), &end, 10);
        p = end;
        (*count)++;
    }
    while (*p && *p != ']') p++;
    return *p ? p + 1 : p;
}

int orc_task_load(const char *path, orc_task_t *spec)
{
    memset(spec, 0, sizeof *spec);
    FILE *f = fopen(path, "rb");
    if (!f) { fprintf(stderr, "Cannot open task file: %s\n", path); return -1; }
    fseek(f, 0, SEEK_END);
    long sz = ftell(f);
    fseek(f, 0, SEEK_SET);
    char *js = malloc((size_t)sz + 1);
    if (!js) { fclose(f); return -1; }
    size_t n = fread(js, 1, (size_t)sz, f);
    js[n] = 0;
    fclose(f);

    const char *p = find_key(js, "name");
    if (p && *p == '"') {
        p++;
        int i = 0;
        while (*p && *p != '"' && i < 63) spec->name[i++] = *p++;
        spec->name[i] = 0;
    }
    p = find_key(js, "max_cycles");
    spec->max_cycles = p ? (uint64_t)strtol(p, NULL, 10) : 1000;
    long v[ORC_MAX_IO_PORTS];
    int cnt;
    if ((p = find_key(js, "input_ports"))) {
        parse_ints(p, v, ORC_MAX_IO_PORTS, &cnt);
        spec->num_inputs = cnt;
        for (int i = 0; i < cnt; i++) spec->input_ports[i] = (uint8_t)v[i];
    }
    if ((p = find_key(js, "output_ports"))) {
        parse_ints(p, v, ORC_MAX_IO_PORTS, &cnt);
        spec->num_outputs = cnt;
        for (int i = 0; i < cnt; i++) spec->output_ports[i] = (uint8_t)v[i];
    }
    if ((p = find_key(js, "tests"))) {
        p = skip_ws(p);
        if (*p == '[') p++;
        while (spec->num_tests < ORC_MAX_TESTS) {
            p = skip_ws(p);
            if (*p == ']' || !*p) break;
            if (*p == ',') p = skip_ws(p + 1);
            if (*p != '{') break;
            const char *obj = p;
            int depth = 1;
            for (p++; *p && depth > 0; p++) {
                if (*p == '{') depth++;
                else if (*p == '}') depth--;
            }
            int t = spec->num_tests;
            const char *q;
            if ((q = find_key(obj, "in"))) {
                parse_ints(q, v, ORC_MAX_IO_PORTS, &cnt);
                for (int i = 0; i < cnt; i++) spec->tests[t].in[i] = (uint16_t)(v[i] & 0xFFFF);
            }
            if ((q = find_key(obj, "out"))) {
                parse_ints(q, v, ORC_MAX_IO_PORTS, &cnt);
                for (int i = 0; i < cnt; i++) spec->tests[t].out[i] = (uint16_t)(v[i] & 0xFFFF);
            }
            spec->num_tests++;
        }
    }
    free(js);
    return 0;
}

/* ---- VM (src/vm.c:28-217) ----------------------------------------------- */

typedef struct {
    uint16_t r[8], mem[256], prog[256], stack[16], ports[8];
    uint8_t pc, sp, flags, status;
    uint64_t cycles;
} orc_vm_t;

static void vm_flags_zn(orc_vm_t *vm, uint16_t r)
{
    vm->flags = (uint8_t)((r == 0 ? F_Z : 0) | (r & 0x8000 ? F_N : 0));
}

static void vm_flags_add(orc_vm_t *vm, uint16_t a, uint16_t b)
{
    uint32_t w = (uint32_t)a + b;
    uint16_t r = (uint16_t)w;
    vm_flags_zn(vm, r);
    if (w > 0xFFFF) vm->flags |= F_C;
    if (~(a ^ b) & (a ^ r) & 0x8000) vm->flags |= F_V;
}

static void vm_flags_sub(orc_vm_t *vm, uint16_t a, uint16_t b)
{
    uint16_t r = (uint16_t)(a - b);
    vm_flags_zn(vm, r);
    if (a >= b) vm->flags |= F_C;
    if ((a ^ b) & (a ^ r) & 0x8000) vm->flags |= F_V;
}

static void vm_step(orc_vm_t *vm)
{
    if (vm->status != 0) return;
    uint16_t in = vm->prog[vm->pc];
    uint8_t op = I_OP(in), rd = I_RD(in), rs = I_RS(in), rt = I_RT(in);
    uint8_t imm = I_IMM(in);
    int8_t simm = (int8_t)imm;
    uint16_t *r = vm->r;
    vm->pc++;
    switch (op) {
    case OP_NOP: break;
    case OP_HLT: vm->status = 1; break;
    case OP_ADD: vm_flags_add(vm, r[rs], r[rt]); r[rd] = (uint16_t)(r[rs] + r[rt]); break;
    case OP_SUB: vm_flags_sub(vm, r[rs], r[rt]); r[rd] = (uint16_t)(r[rs] - r[rt]); break;
    case OP_MUL: {
        uint32_t p = (uint32_t)r[rs] * r[rt];
        r[rd] = (uint16_t)p;
        vm_flags_zn(vm, r[rd]);
        if (p > 0xFFFF) vm->flags |= F_C;
        break;
    }
    case OP_DIV:
        if (!r[rt]) { vm->status = 3; break; }
        r[rd] = (uint16_t)((int16_t)r[rs] / (int16_t)r[rt]);
        vm_flags_zn(vm, r[rd]);
        break;
    case OP_MOD:
        if (!r[rt]) { vm->status = 3; break; }
        r[rd] = (uint16_t)((int16_t)r[rs] % (int16_t)r[rt]);
        vm_flags_zn(vm, r[rd]);
        break;
    case OP_AND: r[rd] = r[rs] & r[rt]; vm_flags_zn(vm, r[rd]); break;
    case OP_OR:  r[rd] = r[rs] | r[rt]; vm_flags_zn(vm, r[rd]); break;
    case OP_XOR: r[rd] = r[rs] ^ r[rt]; vm_flags_zn(vm, r[rd]); break;
    case OP_SHL: r[rd] = (uint16_t)(r[rs] << (r[rt] & 0xF)); vm_flags_zn(vm, r[rd]); break;
    case OP_SHR: r[rd] = (uint16_t)(r[rs] >> (r[rt] & 0xF)); vm_flags_zn(vm, r[rd]); break;
    case OP_ASR: r[rd] = (uint16_t)((int16_t)r[rs] >> (r[rt] & 0xF)); vm_flags_zn(vm, r[rd]); break;
    case OP_CMP: vm_flags_sub(vm, r[rd], r[rs]); break;
    case OP_LD: r[rd] = vm->mem[r[rs] & 0xFF]; break;
    case OP_ST: vm->mem[r[rd] & 0xFF] = r[rs]; break;
    case OP_LDI: r[rd] = imm; break;
    case OP_LUI: r[rd] = (uint16_t)((r[rd] & 0xFF) | ((uint16_t)imm << 8)); break;
    case OP_ADDI:
        vm_flags_add(vm, r[rd], (uint16_t)(int16_t)simm);
        r[rd] = (uint16_t)(r[rd] + (uint16_t)(int16_t)simm);
        break;
    case OP_BR: {
        uint8_t f = vm->flags;
        int take = 0;
        switch (rd) {
        case 0: take = 1; break;
        case 1: take = (f & F_Z) != 0; break;
        case 2: take = (f & F_Z) == 0; break;
        case 3: take = ((f & F_N) != 0) != ((f & F_V) != 0); break;
        case 4: take = ((f & F_N) != 0) == ((f & F_V) != 0); break;
        case 5: take = (f & F_C) == 0; break;
        case 6: take = (f & F_C) != 0; break;
        }
        if (take) vm->pc = (uint8_t)((int)vm->pc + simm);
        break;
    }
    case OP_JMP: vm->pc = (uint8_t)r[rd]; break;
    case OP_CALL:
        if (vm->sp >= 16) { vm->status = 3; break; }
        vm->stack[vm->sp++] = vm->pc;
        vm->pc = (uint8_t)r[rd];
        break;
    case OP_RET:
        if (vm->sp == 0) { vm->status = 3; break; }
        vm->pc = (uint8_t)vm->stack[--vm->sp];
        break;
    case OP_IN: r[rd] = vm->ports[imm & 7]; break;
    case OP_OUT: vm->ports[imm & 7] = r[rd]; break;
    default: vm->status = 3; break;
    }
    r[0] = 0;
    vm->cycles++;
}

int orc_task_evaluate(const orc_task_t *spec, const uint16_t *prog, int len)
{
    int passed = 0;
    for (int t = 0; t < spec->num_tests; t++) {
        orc_vm_t vm;
        memset(&vm, 0, sizeof vm);
        memcpy(vm.prog, prog, (size_t)(len > 256 ? 256 : len) * 2);
        for (int i = 0; i < spec->num_inputs; i++)
            vm.ports[spec->input_ports[i]] = spec->tests[t].in[i];
        while (vm.status == 0 && vm.cycles < spec->max_cycles) vm_step(&vm);
        if (vm.status != 1) continue;
        int ok = 1;
        for (int i = 0; i < spec->num_outputs; i++)
            if (vm.ports[spec->output_ports[i]] != spec->tests[t].out[i]) { ok = 0; break; }
        passed += ok;
    }
    return passed;
}

/* ---- search state (src/search_state.c:15-239) --------------------------- */

int orc_ctx_init(orc_ctx_t *ctx, const orc_task_t *task)
{
    if (task->num_tests > ORC_MAX_TESTS) return -1;
    if (task->num_outputs != 1) return -1;
    if (task->num_inputs > ORC_NUM_REGS - 1) return -1;
    memset(ctx, 0, sizeof *ctx);
    ctx->task = *task;
    ctx->num_tests = (uint8_t)task->num_tests;
    ctx->num_inputs = (uint8_t)task->num_inputs;
    ctx->num_outputs = (uint8_t)task->num_outputs;
    for (int i = 0; i < task->num_inputs; i++) ctx->input_regs[i] = (uint8_t)(i + 1);
    ctx->output_port = task->output_ports[0];
    return 0;
}

void orc_init_root(const orc_ctx_t *ctx, orc_state_t *s)
{
    memset(s, 0, sizeof *s);
    for (int t = 0; t < ctx->num_tests; t++)
        for (int i = 0; i < ctx->num_inputs; i++)
            s->regs[t][i + 1] = ctx->task.tests[t].in[i];
    for (int i = 0; i < ctx->num_inputs; i++) s->live |= (uint8_t)(1u << (i + 1));
}

static uint8_t zn(uint16_t r) { return (uint8_t)((r == 0 ? F_Z : 0) | (r & 0x8000 ? F_N : 0)); }

int orc_step(const orc_ctx_t *ctx, const orc_state_t *src, uint16_t insn, orc_state_t *dst)
{
    uint8_t op = I_OP(insn), rd = I_RD(insn), rs = I_RS(insn), rt = I_RT(insn);
    uint8_t imm = I_IMM(insn);
    switch (op) {
    case OP_ADD: case OP_SUB: case OP_MUL: case OP_DIV: case OP_MOD:
    case OP_AND: case OP_OR: case OP_XOR: case OP_SHL: case OP_SHR:
    case OP_ASR: case OP_LDI: case OP_ADDI: break;
    default: return 0;
    }
    *dst = *src;
    dst->depth = (uint8_t)(src->depth + 1);
    for (int t = 0; t < ctx->num_tests; t++) {
        uint16_t *r = dst->regs[t];
        uint8_t *f = &dst->flags[t];
        uint16_t a = r[rs], b = r[rt], res;
        uint32_t w;
        switch (op) {
        case OP_ADD:
            w = (uint32_t)a + b; res = (uint16_t)w;
            *f = zn(res) | (w > 0xFFFF ? F_C : 0) | ((~(a ^ b) & (a ^ res) & 0x8000) ? F_V : 0);
            r[rd] = res; break;
        case OP_SUB:
            res = (uint16_t)(a - b);
            *f = zn(res) | (a >= b ? F_C : 0) | (((a ^ b) & (a ^ res) & 0x8000) ? F_V : 0);
            r[rd] = res; break;
        case OP_MUL:
            w = (uint32_t)a * b; res = (uint16_t)w;
            *f = zn(res) | (w > 0xFFFF ? F_C : 0);
            r[rd] = res; break;
        case OP_DIV:
            if (!b) return 0;
            r[rd] = (uint16_t)((int16_t)a / (int16_t)b); *f = zn(r[rd]); break;
        case OP_MOD:
            if (!b) return 0;
            r[rd] = (uint16_t)((int16_t)a % (int16_t)b); *f = zn(r[rd]); break;
        case OP_AND: r[rd] = a & b; *f = zn(r[rd]); break;
        case OP_OR:  r[rd] = a | b; *f = zn(r[rd]); break;
        case OP_XOR: r[rd] = a ^ b; *f = zn(r[rd]); break;
        case OP_SHL: r[rd] = (uint16_t)(a << (b & 0xF)); *f = zn(r[rd]); break;
        case OP_SHR: r[rd] = (uint16_t)(a >> (b & 0xF)); *f = zn(r[rd]); break;
        case OP_ASR: r[rd] = (uint16_t)((int16_t)a >> (b & 0xF)); *f = zn(r[rd]); break;
        case OP_LDI: r[rd] = imm; break;            /* flags untouched */
        case OP_ADDI: {
            uint16_t x = r[rd], e = (uint16_t)(int16_t)(int8_t)imm;
            w = (uint32_t)x + e; res = (uint16_t)w;
            *f = zn(res) | (w > 0xFFFF ? F_C : 0) | ((~(x ^ e) & (x ^ res) & 0x8000) ? F_V : 0);
            r[rd] = res; break;
        }
        }
        r[0] = 0;
    }
    if (rd != 0) dst->live = (uint8_t)(src->live | (1u << rd));
    return 1;
}

static uint64_t fnv(uint64_t h, uint8_t b) { return (h ^ b) * 0x00000100000001B3ULL; }

uint64_t orc_oep_hash64(const orc_ctx_t *ctx, const orc_state_t *s)
{
    uint64_t h = 0xCBF29CE484222325ULL;
    for (int t = 0; t < ctx->num_tests; t++) {
        for (int r = 0; r < 8; r++) {
            h = fnv(h, (uint8_t)(s->regs[t][r] & 0xFF));
            h = fnv(h, (uint8_t)(s->regs[t][r] >> 8));
        }
        h = fnv(h, s->flags[t]);
    }
    return h;
}

uint64_t orc_key_hash64(const orc_ctx_t *ctx, const orc_state_t *s)
{
    return fnv(fnv(orc_oep_hash64(ctx, s), s->live), s->depth);
}

uint8_t orc_leaf_outputs(const orc_ctx_t *ctx, const orc_state_t *s)
{
    uint8_t res = 0;
    for (int r = 1; r < 8; r++) {
        if (!(s->live & (1u << r))) continue;
        int ok = 1;
        for (int t = 0; t < ctx->num_tests && ok; t++)
            ok = s->regs[t][r] == ctx->task.tests[t].out[0];
        if (ok) res |= (uint8_t)(1u << r);
    }
    return res;
}

static const uint8_t LDI_VALS[12] = {0, 1, 2, 3, 4, 5, 8, 16, 32, 64, 128, 255};
static const int8_t ADDI_VALS[6] = {-1, 1, -2, 2, -3, 3};

int orc_gen_candidates(uint16_t *out, int max, uint8_t live)
{
    static const uint8_t ops[9] = {OP_ADD, OP_SUB, OP_MUL, OP_AND, OP_OR,
                                   OP_XOR, OP_SHL, OP_SHR, OP_ASR};
    static const int comm[9] = {1, 0, 1, 1, 1, 1, 0, 0, 0};
    int n = 0;
    for (int oi = 0; oi < 9; oi++) {
        int op = ops[oi];
        for (int rd = 1; rd < 8 && n < max; rd++)
            for (int rs = 0; rs < 8 && n < max; rs++) {
                if (rs && !(live & (1 << rs))) continue;
                for (int rt = comm[oi] ? rs : 0; rt < 8 && n < max; rt++) {
                    if (rt && !(live & (1 << rt))) continue;
                    if (rs == 0 && rt == 0) continue;
                    if (op == OP_ADD && rs == rd && rt == 0) continue;
                    if (op == OP_ADD && rt == rd && rs == 0) continue;
                    if (op == OP_SUB && rs == rd && rt == 0) continue;
                    if (op == OP_MUL && (rs == 0 || rt == 0)) continue;
                    if ((op == OP_SHL || op == OP_SHR || op == OP_ASR) && rt == 0) continue;
                    out[n++] = ENC_R(op, rd, rs, rt);
                }
            }
    }
    for (int rd = 1; rd < 8 && n < max; rd++)
        for (int i = 0; i < 12 && n < max; i++) out[n++] = ENC_I(OP_LDI, rd, LDI_VALS[i]);
    for (int rd = 1; rd < 8 && n < max; rd++) {
        if (!(live & (1 << rd))) continue;
        for (int i = 0; i < 6 && n < max; i++) out[n++] = ENC_I(OP_ADDI, rd, (uint8_t)ADDI_VALS[i]);
    }
    return n;
}

/* ---- 32-bit OEP table of the reference (tools/enumerate.c:43-89) -------- */

#define REF_OEP_BITS 20
#define REF_OEP_SIZE (1u << REF_OEP_BITS)

typedef struct { uint32_t *tab[ORC_MAX_DEPTH]; } ref_oep_t;

static int ref_oep_check_insert(ref_oep_t *o, int depth, uint32_t h)
{
    if (!o->tab[depth]) {
        o->tab[depth] = calloc(REF_OEP_SIZE, 4);
        if (!o->tab[depth]) return 0;
    }
    uint32_t key = h | 1, idx = h & (REF_OEP_SIZE - 1);
    for (int p = 0; p < 32; p++) {
        uint32_t *slot = &o->tab[depth][(idx + p) & (REF_OEP_SIZE - 1)];
        if (*slot == 0) { *slot = key; return 0; }
        if (*slot == key) return 1;
    }
    return 0;
}

static void ref_oep_clear(ref_oep_t *o)
{
    for (int d = 0; d < ORC_MAX_DEPTH; d++)
        if (o->tab[d]) memset(o->tab[d], 0, REF_OEP_SIZE * 4);
}

static void ref_oep_free(ref_oep_t *o)
{
    for (int d = 0; d < ORC_MAX_DEPTH; d++) free(o->tab[d]);
}

/* ---- exact-key set (full state bytes compared on every hash hit) -------- */

typedef struct {
    uint64_t *slot;    /* (hash | 1) or 0 */
    uint32_t *ref;     /* index into keys */
    uint8_t  *keys;
    size_t cap, n, keylen, keys_cap;
} exact_set_t;

static size_t exact_key(const orc_ctx_t *ctx, const orc_state_t *s, int with_live, uint8_t *k)
{
    size_t n = 0;
    for (int t = 0; t < ctx->num_tests; t++) {
        memcpy(k + n, s->regs[t], 16);
        n += 16;
    }
    memcpy(k + n, s->flags, ctx->num_tests);
    n += ctx->num_tests;
    if (with_live) k[n++] = s->live;
    return n;
}

static uint64_t bytes_hash(const uint8_t *k, size_t n)
{
    uint64_t h = 0x9E3779B97F4A7C15ULL;
    for (size_t i = 0; i < n; i++) { h ^= k[i]; h *= 0x100000001B3ULL; h ^= h >> 29; }
    return h | 1;
}

static void exact_clear(exact_set_t *e)
{
    if (e->slot) memset(e->slot, 0, e->cap * 8);
    e->n = 0;
}

static void exact_free(exact_set_t *e)
{
    free(e->slot); free(e->ref); free(e->keys);
    memset(e, 0, sizeof *e);
}

static int exact_insert_raw(exact_set_t *e, const uint8_t *k, size_t len, uint64_t h);

static void exact_grow(exact_set_t *e)
{
    size_t oc = e->cap;
    uint64_t *os = e->slot;
    uint32_t *orf = e->ref;
    e->cap = oc ? oc * 2 : (1u << 16);
    e->slot = calloc(e->cap, 8);
    e->ref = calloc(e->cap, 4);
    size_t n = e->n;
    e->n = 0;
    (void)n;
    for (size_t i = 0; i < oc; i++) {
        if (!os[i]) continue;
        size_t j = os[i] & (e->cap - 1);
        while (e->slot[j]) j = (j + 1) & (e->cap - 1);
        e->slot[j] = os[i];
        e->ref[j] = orf[i];
        e->n++;
    }
    free(os);
    free(orf);
}

/* Returns 1 if already present, 0 if newly inserted. */
static int exact_insert_raw(exact_set_t *e, const uint8_t *k, size_t len, uint64_t h)
{
    if ((e->n + 1) * 2 > e->cap) exact_grow(e);
    if (e->keylen != len) e->keylen = len;
    size_t j = h & (e->cap - 1);
    while (e->slot[j]) {
        if (e->slot[j] == h && memcmp(e->keys + (size_t)e->ref[j] * len, k, len) == 0) return 1;
        j = (j + 1) & (e->cap - 1);
    }
    if ((e->n + 1) * len > e->keys_cap) {
        e->keys_cap = e->keys_cap ? e->keys_cap * 2 : (size_t)len * 65536;
        while (e->keys_cap < (e->n + 1) * len) e->keys_cap *= 2;
        e->keys = realloc(e->keys, e->keys_cap);
    }
    memcpy(e->keys + e->n * len, k, len);
    e->slot[j] = h;
    e->ref[j] = (uint32_t)e->n;
    e->n++;
    return 0;
}

/* ---- enumerate (tools/enumerate.c:292-402, 624-662) --------------------- */

typedef struct {
    orc_ctx_t ctx;
    int mode;
    int sol_cap;            /* <0: reference cap 100 with early stop */
    uint16_t program[256];
    uint16_t *sol_progs;
    int *sol_lens;
    int num_stored;
    uint64_t total_sols;
    uint64_t tried, pruned;
    uint64_t false_prunes, missed_prunes;
    ref_oep_t ref;
    exact_set_t ex[ORC_MAX_DEPTH];
    uint64_t survivors[ORC_MAX_DEPTH + 1], children[ORC_MAX_DEPTH + 1];
} orc_solver_t;

static int solver_stopped(const orc_solver_t *s)
{
    return s->sol_cap < 0 && s->total_sols >= 100;
}

/* enumerate.c:292-313 */
static void try_output(orc_solver_t *s, const orc_state_t *st, int kend)
{
    if (solver_stopped(s)) return;
    uint8_t solving = orc_leaf_outputs(&s->ctx, st);
    for (int r = 1; r < 8; r++) {
        if (!(solving & (1u << r))) continue;
        s->program[kend] = ENC_I(OP_OUT, r, s->ctx.task.output_ports[0]);
        s->program[kend + 1] = ENC_R(OP_HLT, 0, 0, 0);
        int plen = kend + 2;
        s->tried++;
        if (orc_task_evaluate(&s->ctx.task, s->program, plen) == s->ctx.task.num_tests) {
            int cap = s->sol_cap < 0 ? 100 : s->sol_cap;
            if (s->num_stored < cap && s->sol_progs) {
                memset(s->sol_progs + (size_t)s->num_stored * 16, 0, 32);
                memcpy(s->sol_progs + (size_t)s->num_stored * 16, s->program,
                       (size_t)(plen > 16 ? 16 : plen) * 2);
                s->sol_lens[s->num_stored] = plen;
                s->num_stored++;
            }
            s->total_sols++;
        }
    }
}

/* returns 1 if the child is pruned */
static int oep_prune(orc_solver_t *s, int pos, const orc_state_t *child)
{
    uint8_t key[ORC_MAX_TESTS * 17 + 1];
    size_t len;
    switch (s->mode) {
    case ORC_OEP_REF32:
        return ref_oep_check_insert(&s->ref, pos, (uint32_t)orc_oep_hash64(&s->ctx, child));
    case ORC_OEP_REF32_AUDIT: {
        int ref = ref_oep_check_insert(&s->ref, pos, (uint32_t)orc_oep_hash64(&s->ctx, child));
        len = exact_key(&s->ctx, child, 0, key);
        int seen = exact_insert_raw(&s->ex[pos], key, len, bytes_hash(key, len));
        if (ref && !seen) s->false_prunes++;
        if (!ref && seen) s->missed_prunes++;
        return ref;
    }
    case ORC_OEP_EXACT:
    case ORC_OEP_EXACT_LIVE:
        len = exact_key(&s->ctx, child, s->mode == ORC_OEP_EXACT_LIVE, key);
        return exact_insert_raw(&s->ex[pos], key, len, bytes_hash(key, len));
    default:
        return 0;
    }
}

/* enumerate.c:316-402 (branchless search_state DFS, recorder omitted) */
static void dfs(orc_solver_t *s, const orc_state_t *st, int pos, int K)
{
    if (solver_stopped(s)) return;
    int kstart = s->ctx.num_inputs;
    if (pos == K) {
        try_output(s, st, kstart + K);
        return;
    }
    uint16_t cands[4096];
    int nc = orc_gen_candidates(cands, 4096, st->live);
    for (int i = 0; i < nc; i++) {
        if (solver_stopped(s)) return;
        orc_state_t child;
        if (!orc_step(&s->ctx, st, cands[i], &child)) continue;
        s->program[kstart + pos] = cands[i];
        s->tried++;
        s->children[pos + 1]++;
        if (oep_prune(s, pos, &child)) { s->pruned++; continue; }
        s->survivors[pos + 1]++;
        dfs(s, &child, pos + 1, K);
    }
}

static void solver_setup(orc_solver_t *s, const orc_task_t *task)
{
    orc_ctx_init(&s->ctx, task);
    for (int i = 0; i < task->num_inputs; i++)
        s->program[i] = ENC_I(OP_IN, i + 1, task->input_ports[i]);
}

static void solver_clear_tables(orc_solver_t *s)
{
    ref_oep_clear(&s->ref);
    for (int d = 0; d < ORC_MAX_DEPTH; d++) exact_clear(&s->ex[d]);
}

static void solver_free(orc_solver_t *s)
{
    ref_oep_free(&s->ref);
    for (int d = 0; d < ORC_MAX_DEPTH; d++) exact_free(&s->ex[d]);
}

int orc_enumerate(const orc_task_t *task, int max_depth, int oep_mode, int sol_cap,
                  uint16_t *sol_progs, int *sol_lens, orc_result_t *res)
{
    memset(res, 0, sizeof *res);
    res->optimal_depth = -1;
    if (task->num_outputs != 1 || task->num_tests > ORC_MAX_TESTS ||
        task->num_inputs > 7 || max_depth > ORC_MAX_DEPTH - 1)
        return -1;
    orc_solver_t *s = calloc(1, sizeof *s);
    if (!s) return -1;
    solver_setup(s, task);
    s->mode = oep_mode;
    s->sol_cap = sol_cap;
    s->sol_progs = sol_progs;
    s->sol_lens = sol_lens;
    orc_state_t root;
    orc_init_root(&s->ctx, &root);
    for (int K = 0; K <= max_depth; K++) {
        uint64_t tried0 = s->tried;
        uint64_t sols0 = s->total_sols;
        solver_clear_tables(s);
        memset(s->survivors, 0, sizeof s->survivors);
        memset(s->children, 0, sizeof s->children);
        s->survivors[0] = 1;
        s->children[0] = 1;
        dfs(s, &root, 0, K);
        res->tried[K] = s->tried - tried0;
        res->pruned_cum[K] = s->pruned;
        res->sols_at[K] = (int)(s->total_sols - sols0);
        if (s->total_sols > 0) {
            res->optimal_depth = K;
            break;
        }
    }
    memcpy(res->survivors, s->survivors, sizeof s->survivors);
    memcpy(res->children, s->children, sizeof s->children);
    res->num_solutions = s->num_stored;
    res->total_solutions = s->total_sols;
    res->false_prunes = s->false_prunes;
    res->missed_prunes = s->missed_prunes;
    solver_free(s);
    free(s);
    return 0;
}

/* ---- exhaustive completion (src/search_state.c:339-453) ----------------- */

typedef struct {
    const orc_ctx_t *ctx;
    ref_oep_t oep;
    uint64_t explored;
} exh_t;

static int exh_dfs(exh_t *e, const orc_state_t *s, int pos, int target, uint16_t *path)
{
    uint16_t cands[4096];
    int nc = orc_gen_candidates(cands, 4096, s->live);
    for (int i = 0; i < nc; i++) {
        orc_state_t child;
        if (!orc_step(e->ctx, s, cands[i], &child)) continue;
        e->explored++;
        if (orc_leaf_outputs(e->ctx, &child)) { path[pos] = cands[i]; return pos + 1; }
        if (pos + 1 >= target) continue;
        if (ref_oep_check_insert(&e->oep, pos, (uint32_t)orc_oep_hash64(e->ctx, &child))) continue;
        path[pos] = cands[i];
        int len = exh_dfs(e, &child, pos + 1, target, path);
        if (len > 0) return len;
    }
    return 0;
}

int orc_exhaustive_complete(const orc_ctx_t *ctx, const orc_state_t *start, int max_depth,
                            uint16_t *sol, int *sol_len, uint64_t *states_explored)
{
    exh_t e;
    memset(&e, 0, sizeof e);
    e.ctx = ctx;
    *sol_len = 0;
    int found = 0;
    if (orc_leaf_outputs(ctx, start)) {
        found = 1;
    } else {
        int max_r = max_depth - (int)start->depth;
        if (max_r > ORC_MAX_DEPTH) max_r = ORC_MAX_DEPTH;
        uint16_t path[ORC_MAX_DEPTH];
        for (int target = 1; target <= max_r && !found; target++) {
            ref_oep_clear(&e.oep);
            int len = exh_dfs(&e, start, 0, target, path);
            if (len > 0) {
                memcpy(sol, path, (size_t)len * 2);
                *sol_len = len;
                found = 1;
            }
        }
    }
    if (states_explored) *states_explored = e.explored;
    ref_oep_free(&e.oep);
    return found;
}

/* ---- threaded CPU sample ------------------------------------------------ */

typedef struct {
    const orc_task_t *task;
    int depth;
    double budget;            /* seconds; no new work item after this */
    volatile long *next;      /* shared work-item counter */
    struct timespec t0;
    uint64_t tried, sols;
} sample_arg_t;

static double since(const struct timespec *t0)
{
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)(t.tv_sec - t0->tv_sec) + 1e-9 * (double)(t.tv_nsec - t0->tv_nsec);
}

/* ---- branch mode (tools/enumerate.c:204-286, 405-455, 624-662) --------- */

/* Candidates of a position (tools/enumerate.c:204-260): ALU ops with DIV and
   MOD, CMP, forward BR (cond 1..6, offset 1..kernel_depth - pos - 1), LDI,
   ADDI, in the reference's order. */
static int gen_branch_candidates(uint16_t *out, int max, uint8_t live, int pos, int kdepth)
{
    static const uint8_t alu[] = {OP_ADD, OP_SUB, OP_MUL, OP_DIV, OP_MOD,
                                  OP_AND, OP_OR, OP_XOR, OP_SHL, OP_SHR, OP_ASR};
    static const int commut[] = {1, 0, 1, 0, 0, 1, 1, 1, 0, 0, 0};
    int n = 0;
    for (int oi = 0; oi < 11; oi++) {
        const int op = alu[oi];
        for (int rd = 1; rd < 8 && n < max; rd++)
            for (int rs = 0; rs < 8 && n < max; rs++) {
                if (rs && !(live >> rs & 1)) continue;
                for (int rt = commut[oi] ? rs : 0; rt < 8 && n < max; rt++) {
                    if (rt && !(live >> rt & 1)) continue;
                    if (rs == 0 && rt == 0) continue;
                    if (op == OP_ADD && rs == rd && rt == 0) continue;
                    if (op == OP_ADD && rt == rd && rs == 0) continue;
                    if (op == OP_SUB && rs == rd && rt == 0) continue;
                    if (op == OP_MUL && (rs == 0 || rt == 0)) continue;
                    if ((op == OP_DIV || op == OP_MOD) && rt == 0) continue;
                    if ((op == OP_SHL || op == OP_SHR || op == OP_ASR) && rt == 0) continue;
                    out[n++] = ENC_R(op, rd, rs, rt);
                }
            }
    }
    for (int rd = 0; rd < 8 && n < max; rd++) {
        if (rd && !(live >> rd & 1)) continue;
        for (int rs = 0; rs < 8 && n < max; rs++) {
            if (rs && !(live >> rs & 1)) continue;
            if ((rd == 0 && rs == 0) || rd == rs) continue;
            out[n++] = ENC_R(OP_CMP, rd, rs, 0);
        }
    }
    const int mf = kdepth - pos - 1;
    for (int cond = 1; cond <= 6 && mf > 0; cond++)
        for (int off = 1; off <= mf && n < max; off++) out[n++] = ENC_I(OP_BR, cond, (uint8_t)off);
    for (int rd = 1; rd < 8 && n < max; rd++)
        for (int i = 0; i < 12 && n < max; i++) out[n++] = ENC_I(OP_LDI, rd, LDI_VALS[i]);
    for (int rd = 1; rd < 8 && n < max; rd++) {
        if (!(live >> rd & 1)) continue;
        for (int i = 0; i < 6 && n < max; i++) out[n++] = ENC_I(OP_ADDI, rd, (uint8_t)ADDI_VALS[i]);
    }
    return n;
}

typedef struct {
    const orc_task_t *task;
    int mode, num_inputs;
    uint16_t program[256];
    uint16_t *sol_progs;
    int *sol_lens;
    int num_solutions;
    uint64_t tried, pruned;
    ref_oep_t ref;
    exact_set_t ex[ORC_MAX_DEPTH];
} bsolver_t;

static void branch_try_output(bsolver_t *s, uint8_t live, int kend)
{
    if (s->num_solutions >= 100) return;
    for (int r = 1; r < 8; r++) {
        if (!(live >> r & 1)) continue;
        s->program[kend] = ENC_I(OP_OUT, r, s->task->output_ports[0]);
        s->program[kend + 1] = ENC_R(OP_HLT, 0, 0, 0);
        s->tried++;
        if (orc_task_evaluate(s->task, s->program, kend + 2) == s->task->num_tests) {
            if (s->sol_progs && s->num_solutions < 100) {
                memset(s->sol_progs + (size_t)s->num_solutions * 16, 0, 32);
                memcpy(s->sol_progs + (size_t)s->num_solutions * 16, s->program, (size_t)(kend + 2) * 2);
                s->sol_lens[s->num_solutions] = kend + 2;
            }
            s->num_solutions++;
        }
    }
}

static void branch_dfs(bsolver_t *s, int pos, int kdepth, uint8_t live)
{
    if (s->num_solutions >= 100) return;
    const int kstart = s->num_inputs;
    if (pos == kdepth) {
        branch_try_output(s, live, kstart + kdepth);
        return;
    }
    uint16_t cands[4096];
    const int nc = gen_branch_candidates(cands, 4096, live, pos, kdepth);
    const int ppos = kstart + pos;
    for (int i = 0; i < nc; i++) {
        if (s->num_solutions >= 100) return;
        s->program[ppos] = cands[i];
        const uint8_t op = I_OP(cands[i]), rd = I_RD(cands[i]);
        uint8_t nl = live;
        if (op != OP_CMP && op != OP_BR && rd != 0) nl |= (uint8_t)(1u << rd);
        if (s->mode != ORC_OEP_NONE && op != OP_BR) {
            /* the partial program, HLT appended, on every test (100 cycles) */
            const int plen = ppos + 1;
            s->program[plen] = ENC_R(OP_HLT, 0, 0, 0);
            uint32_t h = 2166136261u;
            uint8_t key[ORC_MAX_TESTS * 17];
            size_t kn = 0;
            for (int t = 0; t < s->task->num_tests; t++) {
                orc_vm_t vm;
                memset(&vm, 0, sizeof vm);
                memcpy(vm.prog, s->program, (size_t)(plen + 1) * 2);
                for (int p = 0; p < s->task->num_inputs; p++)
                    vm.ports[s->task->input_ports[p]] = s->task->tests[t].in[p];
                while (vm.status == 0 && vm.cycles < 100) vm_step(&vm);
                for (int r = 0; r < 8; r++) {
                    h ^= vm.r[r] & 0xFF; h *= 16777619u;
                    h ^= vm.r[r] >> 8;   h *= 16777619u;
                    memcpy(key + kn, &vm.r[r], 2);
                    kn += 2;
                }
                h ^= vm.flags; h *= 16777619u;
                key[kn++] = vm.flags;
            }
            int seen;
            if (s->mode == ORC_OEP_REF32) seen = ref_oep_check_insert(&s->ref, pos, h);
            else seen = exact_insert_raw(&s->ex[pos], key, kn, bytes_hash(key, kn));
            if (seen) {
                s->pruned++;
                continue;
            }
        }
        s->tried++;
        branch_dfs(s, pos + 1, kdepth, nl);
    }
}

int orc_enumerate_branch(const orc_task_t *task, int max_depth, int oep_mode,
                         uint16_t *sol_progs, int *sol_lens, orc_result_t *res)
{
    memset(res, 0, sizeof *res);
    res->optimal_depth = -1;
    if (task->num_outputs != 1 || task->num_tests > ORC_MAX_TESTS || max_depth < 0 ||
        task->num_inputs + max_depth + 2 > 16)
        return -1;
    bsolver_t *s = calloc(1, sizeof *s);
    if (!s) return -1;
    s->task = task;
    s->mode = oep_mode == ORC_OEP_REF32 || oep_mode == ORC_OEP_NONE ? oep_mode : ORC_OEP_EXACT;
    s->num_inputs = task->num_inputs;
    s->sol_progs = sol_progs;
    s->sol_lens = sol_lens;
    uint8_t live0 = 0;
    for (int i = 0; i < task->num_inputs; i++) {
        s->program[i] = ENC_I(OP_IN, i + 1, task->input_ports[i]);
        live0 |= (uint8_t)(1u << (i + 1));
    }
    for (int K = 0; K <= max_depth; K++) {
        const uint64_t tried0 = s->tried;
        ref_oep_clear(&s->ref);
        for (int d = 0; d < ORC_MAX_DEPTH; d++) exact_clear(&s->ex[d]);
        branch_dfs(s, 0, K, live0);
        res->tried[K] = s->tried - tried0;
        res->pruned_cum[K] = s->pruned;
        res->sols_at[K] = s->num_solutions;
        if (s->num_solutions > 0) {
            res->optimal_depth = K;
            break;
        }
    }
    res->num_solutions = s->num_solutions < 100 ? s->num_solutions : 100;
    res->total_solutions = (uint64_t)s->num_solutions;
    ref_oep_free(&s->ref);
    for (int d = 0; d < ORC_MAX_DEPTH; d++) exact_free(&s->ex[d]);
    free(s);
    return 0;
}

/* Work item k = (root candidate k / 4096, level-1 candidate k % 4096): the
 * thread steps both instructions (counting them as the reference does) and
 * runs the reference DFS below, with its own 32-bit OEP tables kept across
 * its items. */
static void *sample_worker(void *p)
{
    sample_arg_t *a = p;
    orc_solver_t *s = calloc(1, sizeof *s);
    if (!s) return NULL;
    solver_setup(s, a->task);
    s->mode = ORC_OEP_REF32;
    s->sol_cap = 0;
    orc_state_t root;
    orc_init_root(&s->ctx, &root);
    uint16_t c0[4096], c1[4096];
    int n0 = orc_gen_candidates(c0, 4096, root.live);
    for (;;) {
        if (since(&a->t0) > a->budget) break;
        long k = __sync_fetch_and_add(a->next, 1L);
        long i = k / 4096, j = k % 4096;
        if (i >= n0) break;
        orc_state_t s1, s2;
        if (!orc_step(&s->ctx, &root, c0[i], &s1)) continue;
        if (j == 0) s->tried++;
        if (a->depth < 2) continue;
        int n1 = orc_gen_candidates(c1, 4096, s1.live);
        if (j >= n1) continue;
        if (!orc_step(&s->ctx, &s1, c1[j], &s2)) continue;
        s->tried++;
        s->program[s->ctx.num_inputs] = c0[i];
        s->program[s->ctx.num_inputs + 1] = c1[j];
        dfs(s, &s2, 2, a->depth);
    }
    a->tried = s->tried;
    a->sols = s->total_sols;
    solver_free(s);
    free(s);
    return NULL;
}

uint64_t orc_enumerate_sample(const orc_task_t *task, int depth, int nthreads, double budget_s,
                              double *seconds, uint64_t *solutions)
{
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    sample_arg_t args[256];
    volatile long next = 0;
    struct timespec t0;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    for (int i = 0; i < nthreads; i++) {
        args[i] = (sample_arg_t){task, depth, budget_s, &next, t0, 0, 0};
        pthread_create(&th[i], NULL, sample_worker, &args[i]);
    }
    uint64_t tried = 0, sols = 0;
    for (int i = 0; i < nthreads; i++) {
        pthread_join(th[i], NULL);
        tried += args[i].tried;
        sols += args[i].sols;
    }
    if (seconds) *seconds = since(&t0);
    if (solutions) *solutions = sols;
    return tried;
}
