/*
 * host_abi.cpp -- the host half of libpcagb.so: the reference libpca.so ABI
 * (VM, task JSON, search-state primitives) and the candidate tables the GPU
 * engine uploads.
 *
 * Behaviour follows the reference functions cited on each definition; the
 * code is this project's own.
 */
#include "../../include/pca_gb300.h"
#include "gen_tables.h"
#include "pca_isa.h"

#include <algorithm>
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>

namespace pcagb {

static const uint8_t kLdiImm[12] = {0, 1, 2, 3, 4, 5, 8, 16, 32, 64, 128, 255};
static const int8_t kAddiImm[6] = {-1, 1, -2, 2, -3, 3};

/* src/search_state.c:280-330 */
int gen_candidates(uint8_t live, uint16_t *out, int max)
{
    struct AluOp { uint32_t op; bool commutes; };
    static const AluOp ops[9] = {
        {PCA_OP_ADD, true}, {PCA_OP_SUB, false}, {PCA_OP_MUL, true},
        {PCA_OP_AND, true}, {PCA_OP_OR, true},   {PCA_OP_XOR, true},
        {PCA_OP_SHL, false}, {PCA_OP_SHR, false}, {PCA_OP_ASR, false}};
    auto usable = [live](uint32_t r) { return r == 0 || (live >> r) & 1u; };
    int n = 0;
    for (const AluOp &o : ops) {
        for (uint32_t rd = 1; rd < 8; rd++)
            for (uint32_t rs = 0; rs < 8; rs++) {
                if (!usable(rs)) continue;
                for (uint32_t rt = o.commutes ? rs : 0; rt < 8; rt++) {
                    if (!usable(rt) || (rs == 0 && rt == 0)) continue;
                    bool noop = (o.op == PCA_OP_ADD && rt == 0 && rs == rd) ||
                                (o.op == PCA_OP_ADD && rs == 0 && rt == rd) ||
                                (o.op == PCA_OP_SUB && rt == 0 && rs == rd) ||
                                (o.op == PCA_OP_MUL && (rs == 0 || rt == 0)) ||
                                ((o.op == PCA_OP_SHL || o.op == PCA_OP_SHR ||
                                  o.op == PCA_OP_ASR) && rt == 0);
                    if (noop) continue;
                    if (n < max) out[n] = PCA_ENC_R(o.op, rd, rs, rt);
                    n++;
                }
            }
    }
    for (uint32_t rd = 1; rd < 8; rd++)
        for (uint8_t imm : kLdiImm) {
            if (n < max) out[n] = PCA_ENC_I(PCA_OP_LDI, rd, imm);
            n++;
        }
    for (uint32_t rd = 1; rd < 8; rd++) {
        if (!((live >> rd) & 1u)) continue;
        for (int8_t imm : kAddiImm) {
            if (n < max) out[n] = PCA_ENC_I(PCA_OP_ADDI, rd, (uint8_t)imm);
            n++;
        }
    }
    return n < max ? n : max;
}

static GenTables build_tables()
{
    GenTables t;
    t.cand_off.assign(129, 0);
    t.vc_off.assign(129, 0);
    uint16_t buf[4096];
    for (int m = 0; m < 128; m++) {
        uint8_t live = (uint8_t)(m << 1);
        int n = gen_candidates(live, buf, 4096);
        t.cand_off[m] = (uint32_t)t.cand.size();
        t.vc_off[m] = (uint32_t)t.vc_uop.size();
        std::vector<uint32_t> classes;
        for (int i = 0; i < n; i++) {
            uint32_t u = pca_uop_from_insn(buf[i]);
            uint32_t key = UOP_OP(u) == PCA_OP_ADDI ? u : (u & ~(7u << 5));
            int ci = -1;
            for (size_t k = 0; k < classes.size(); k++)
                if (classes[k] == key) { ci = (int)k; break; }
            if (ci < 0) { ci = (int)classes.size(); classes.push_back(key); }
            t.cand.push_back(buf[i]);
            t.cand_uop.push_back(u);
            t.cand_vc.push_back((uint16_t)ci);
        }
        for (uint32_t c : classes) t.vc_uop.push_back(c);
        if (n > t.max_nc) t.max_nc = n;
        if ((int)classes.size() > t.max_nvc) t.max_nvc = (int)classes.size();
    }
    t.cand_off[128] = (uint32_t)t.cand.size();
    t.vc_off[128] = (uint32_t)t.vc_uop.size();
    t.chunk_off.assign(129, 0);
    for (int m = 0; m < 128; m++) {
        t.chunk_off[m] = (uint32_t)t.chunks.size();
        const uint32_t base = t.cand_off[m], n = t.cand_off[m + 1] - base;
        uint32_t s = 0;
        while (s < n) {
            uint32_t e = s;
            while (e < n && e - s < 32 && UOP_OP(t.cand_uop[base + e]) == UOP_OP(t.cand_uop[base + s])) e++;
            t.chunks.push_back(s << 8 | (e - s));
            s = e;
        }
    }
    t.chunk_off[128] = (uint32_t)t.chunks.size();
    for (int s = 0; s < 5; s++) t.f[s].assign(128, 0);
    for (int m = 0; m < 128; m++) t.f[0][m] = 1;
    for (int s = 1; s < 5; s++)
        for (int m = 0; m < 128; m++) {
            uint64_t sum = 0;
            for (uint32_t i = t.cand_off[m]; i < t.cand_off[m + 1]; i++) {
                uint32_t rd = UOP_RD(t.cand_uop[i]);
                sum += t.f[s - 1][(m | (1u << (rd - 1))) & 127];
            }
            t.f[s][m] = sum;
        }
    t.vcr_off.assign(128 * 8 + 1, 0);
    for (int m = 0; m < 128; m++)
        for (uint32_t r = 0; r < 8; r++) {
            t.vcr_off[m * 8 + r] = (uint32_t)t.vcr.size();
            if (r == 0) continue;
            for (uint32_t i = t.vc_off[m]; i < t.vc_off[m + 1]; i++) {
                const uint32_t u = t.vc_uop[i];
                if (UOP_A(u) == r || UOP_B(u) == r) t.vcr.push_back((uint16_t)(i - t.vc_off[m]));
            }
        }
    t.vcr_off[128 * 8] = (uint32_t)t.vcr.size();
    /* same-value-and-flags families among one mask's candidates:
       copy of x (ADD rd,r0,x; AND rd,x,x; OR rd,r0,x; OR rd,x,x; XOR rd,r0,x:
       value x, flags Z/N of x), zero with Z (AND rd,r0,x; XOR rd,x,x;
       SHL/SHR/ASR rd,r0,x) and zero with Z and C (SUB rd,x,x), x >= 1 */
    t.cand_dupe.assign(t.cand_uop.size(), 0);
    for (int m = 0; m < 128; m++) {
        std::vector<uint32_t> seen;
        for (uint32_t i = t.cand_off[m]; i < t.cand_off[m + 1]; i++) {
            const uint32_t u = t.cand_uop[i], op = UOP_OP(u), rd = UOP_RD(u);
            const uint32_t a = UOP_A(u), b = UOP_B(u);
            uint32_t key = 0;
            if ((op == PCA_OP_ADD || op == PCA_OP_OR || op == PCA_OP_XOR) && a == 0 && b >= 1)
                key = 1u << 16 | rd << 8 | b;                       /* copy of b */
            else if ((op == PCA_OP_AND || op == PCA_OP_OR) && a == b && a >= 1)
                key = 1u << 16 | rd << 8 | a;                       /* copy of a */
            else if ((op == PCA_OP_AND || op == PCA_OP_SHL || op == PCA_OP_SHR ||
                      op == PCA_OP_ASR) && a == 0 && b >= 1)
                key = 2u << 16 | rd << 8;                           /* zero, Z */
            else if (op == PCA_OP_XOR && a == b && a >= 1)
                key = 2u << 16 | rd << 8;                           /* zero, Z */
            else if (op == PCA_OP_SUB && a == b && a >= 1)
                key = 3u << 16 | rd << 8;                           /* zero, Z and C */
            if (!key) continue;
            if (std::find(seen.begin(), seen.end(), key) != seen.end()) t.cand_dupe[i] = 1;
            else seen.push_back(key);
        }
    }
    t.pr_off.assign(128 * 8 + 1, 0);
    for (int m = 0; m < 128; m++)
        for (uint32_t r = 0; r < 8; r++) {
            t.pr_off[m * 8 + r] = (uint32_t)t.pr.size();
            if (r == 0) continue;
            const size_t first = t.pr.size();
            for (uint32_t i = t.vc_off[m]; i < t.vc_off[m + 1]; i++) {
                const uint32_t u = t.vc_uop[i], op = UOP_OP(u);
                const uint32_t a = UOP_A(u), b = UOP_B(u);
                if (a != r && b != r) continue;
                const uint16_t ci = (uint16_t)(i - t.vc_off[m]);
                if (op == PCA_OP_ADDI) {
                    t.pr.push_back(a | (1u << 15) | (UOP_IMM(u) << 16));
                    t.pr_cls.insert(t.pr_cls.end(), 10, 0xFFFF);
                    t.pr_cls.back() = ci;
                    continue;
                }
                int k = 0;
                while (k < 9 && kPairOps[k] != op) k++;
                if (k == 9) continue;  /* LDI reads no register */
                size_t e = first;
                while (e < t.pr.size() &&
                       ((t.pr[e] & 63u) != (a | (b << 3)) || (t.pr[e] >> 15 & 1u)))
                    e++;
                if (e == t.pr.size()) {
                    t.pr.push_back(a | (b << 3));
                    t.pr_cls.insert(t.pr_cls.end(), 10, 0xFFFF);
                }
                t.pr[e] |= 1u << (6 + k);
                t.pr_cls[e * 10 + k] = ci;
            }
        }
    t.pr_off[128 * 8] = (uint32_t)t.pr.size();
    t.pr_ev.assign(128 * 8, 0);
    for (int i = 0; i < 128 * 8; i++)
        for (uint32_t e = t.pr_off[i]; e < t.pr_off[i + 1]; e++)
            t.pr_ev[i] += (uint32_t)__builtin_popcount((t.pr[e] >> 6) & 0x3FFu);
    for (int s = 0; s < 5; s++) t.ev[s].assign(128, 0);
    for (int m = 0; m < 128; m++) t.ev[1][m] = t.vc_off[m + 1] - t.vc_off[m];
    for (int s = 2; s < 5; s++)
        for (int m = 0; m < 128; m++) {
            uint64_t sum = 0;
            for (uint32_t i = t.cand_off[m]; i < t.cand_off[m + 1]; i++) {
                uint32_t rd = UOP_RD(t.cand_uop[i]);
                sum += t.ev[s - 1][(m | (1u << (rd - 1))) & 127];
            }
            t.ev[s][m] = sum;
        }
    return t;
}

const GenTables &gen_tables()
{
    static GenTables *tables = nullptr;
    static std::once_flag once;
    std::call_once(once, [] { tables = new GenTables(build_tables()); });
    return *tables;
}

}  // namespace pcagb

using namespace pcagb;

extern "C" {

/* ---- VM: src/vm.c:14-217 -------------------------------------------------- */

void pca_init(pca_vm_t *vm) { memset(vm, 0, sizeof *vm); }

void pca_load(pca_vm_t *vm, const uint16_t *prog, size_t len)
{
    if (len > PCA_PROG_SIZE) len = PCA_PROG_SIZE;
    memcpy(vm->prog, prog, len * sizeof(uint16_t));
}

static void vm_set_add_flags(pca_vm_t *vm, uint32_t a, uint32_t b)
{
    uint32_t r = (a + b) & 0xFFFFu;
    vm->flags = (uint8_t)pca_alu_flags(PCA_OP_ADD, a, b, 0, r, 0);
}

static void vm_set_sub_flags(pca_vm_t *vm, uint32_t a, uint32_t b)
{
    uint32_t r = (a - b) & 0xFFFFu;
    vm->flags = (uint8_t)pca_alu_flags(PCA_OP_SUB, a, b, 0, r, 0);
}

void pca_step(pca_vm_t *vm)
{
    if (vm->status != PCA_RUNNING) return;
    uint32_t insn = vm->prog[vm->pc];
    uint32_t op = PCA_INSN_OP(insn), rd = PCA_INSN_RD(insn);
    uint32_t rs = PCA_INSN_RS(insn), rt = PCA_INSN_RT(insn), imm = PCA_INSN_IMM(insn);
    int32_t simm = (int8_t)(uint8_t)imm;
    uint16_t *r = vm->r;
    vm->pc++;
    switch (op) {
    case PCA_OP_NOP: break;
    case PCA_OP_HLT: vm->status = PCA_HALTED; break;
    case PCA_OP_ADD: vm_set_add_flags(vm, r[rs], r[rt]); r[rd] = (uint16_t)(r[rs] + r[rt]); break;
    case PCA_OP_SUB: vm_set_sub_flags(vm, r[rs], r[rt]); r[rd] = (uint16_t)(r[rs] - r[rt]); break;
    case PCA_OP_MUL: {
        uint32_t a = r[rs], b = r[rt];
        r[rd] = (uint16_t)(a * b);
        vm->flags = (uint8_t)pca_alu_flags(PCA_OP_MUL, a, b, 0, r[rd], 0);
        break;
    }
    case PCA_OP_DIV:
    case PCA_OP_MOD:
        if (r[rt] == 0) { vm->status = PCA_FAULT; break; }
        r[rd] = op == PCA_OP_DIV ? (uint16_t)((int16_t)r[rs] / (int16_t)r[rt])
                                 : (uint16_t)((int16_t)r[rs] % (int16_t)r[rt]);
        vm->flags = (uint8_t)pca_zn(r[rd]);
        break;
    case PCA_OP_AND: case PCA_OP_OR: case PCA_OP_XOR:
    case PCA_OP_SHL: case PCA_OP_SHR: case PCA_OP_ASR:
        r[rd] = (uint16_t)pca_alu(op, r[rs], r[rt], 0);
        vm->flags = (uint8_t)pca_zn(r[rd]);
        break;
    case PCA_OP_CMP: vm_set_sub_flags(vm, r[rd], r[rs]); break;
    case PCA_OP_LD: r[rd] = vm->mem[r[rs] & 0xFF]; break;
    case PCA_OP_ST: vm->mem[r[rd] & 0xFF] = r[rs]; break;
    case PCA_OP_LDI: r[rd] = (uint16_t)imm; break;
    case PCA_OP_LUI: r[rd] = (uint16_t)((r[rd] & 0xFF) | (imm << 8)); break;
    case PCA_OP_ADDI:
        vm_set_add_flags(vm, r[rd], (uint16_t)simm);
        r[rd] = (uint16_t)(r[rd] + simm);
        break;
    case PCA_OP_BR: {
        uint32_t f = vm->flags;
        bool n = f & PCA_FN, v = f & PCA_FV;
        bool take = rd == 0 ? true : rd == 1 ? (f & PCA_FZ) : rd == 2 ? !(f & PCA_FZ)
                  : rd == 3 ? (n != v) : rd == 4 ? (n == v) : rd == 5 ? !(f & PCA_FC)
                  : rd == 6 ? (bool)(f & PCA_FC) : false;
        if (take) vm->pc = (uint8_t)((int)vm->pc + simm);
        break;
    }
    case PCA_OP_JMP: vm->pc = (uint8_t)r[rd]; break;
    case PCA_OP_CALL:
        if (vm->sp >= PCA_STACK_DEPTH) { vm->status = PCA_FAULT; break; }
        vm->stack[vm->sp++] = vm->pc;
        vm->pc = (uint8_t)r[rd];
        break;
    case PCA_OP_RET:
        if (vm->sp == 0) { vm->status = PCA_FAULT; break; }
        vm->pc = (uint8_t)vm->stack[--vm->sp];
        break;
    case PCA_OP_IN:
        if (vm->on_read) vm->on_read(vm, (uint8_t)(imm & 7));
        r[rd] = vm->ports[imm & 7];
        break;
    case PCA_OP_OUT:
        vm->ports[imm & 7] = r[rd];
        if (vm->on_write) vm->on_write(vm, (uint8_t)(imm & 7), r[rd]);
        break;
    default: vm->status = PCA_FAULT; break;
    }
    r[0] = 0;
    vm->cycles++;
}

int pca_run(pca_vm_t *vm, uint64_t max_cycles)
{
    while (vm->status == PCA_RUNNING && vm->cycles < max_cycles) pca_step(vm);
    if (vm->status == PCA_RUNNING) vm->status = PCA_TIMEOUT;
    return vm->status;
}

/* src/asm.c:404-503 (text format of the disassembler) */
void pca_disasm(uint16_t insn, char *buf, size_t len)
{
    static const char *names[] = {"NOP", "HLT", "ADD", "SUB", "MUL", "DIV", "MOD", "AND",
                                  "OR", "XOR", "SHL", "SHR", "ASR", "CMP", "LD", "ST",
                                  "LDI", "LUI", "ADDI", "BR", "JMP", "CALL", "RET", "IN", "OUT"};
    static const char *conds[] = {"BRA", "BZ", "BNZ", "BLT", "BGE", "BLTU", "BGEU"};
    unsigned op = PCA_INSN_OP(insn), rd = PCA_INSN_RD(insn), rs = PCA_INSN_RS(insn);
    unsigned rt = PCA_INSN_RT(insn), imm = PCA_INSN_IMM(insn);
    int simm = (int8_t)(uint8_t)imm;
    if (op > PCA_OP_OUT) { snprintf(buf, len, "??? 0x%04X", insn); return; }
    switch (op) {
    case PCA_OP_NOP: case PCA_OP_HLT: case PCA_OP_RET:
        snprintf(buf, len, "%s", names[op]); break;
    case PCA_OP_CMP: case PCA_OP_LD: case PCA_OP_ST:
        snprintf(buf, len, "%-4s r%u, r%u", names[op], rd, rs); break;
    case PCA_OP_JMP: case PCA_OP_CALL:
        snprintf(buf, len, "%-4s r%u", names[op], rd); break;
    case PCA_OP_LDI: snprintf(buf, len, "LDI  r%u, %u", rd, imm); break;
    case PCA_OP_LUI: snprintf(buf, len, "LUI  r%u, 0x%02X", rd, imm); break;
    case PCA_OP_ADDI: snprintf(buf, len, "ADDI r%u, %d", rd, simm); break;
    case PCA_OP_BR:
        if (rd < 7) snprintf(buf, len, "%-4s %+d", conds[rd], simm);
        else snprintf(buf, len, "BR   %u, %+d", rd, simm);
        break;
    case PCA_OP_IN: case PCA_OP_OUT:
        snprintf(buf, len, "%-4s r%u, %u", names[op], rd, imm & 7); break;
    default:
        if (op == PCA_OP_ADD && rt == 0) snprintf(buf, len, "MOV  r%u, r%u", rd, rs);
        else if (op == PCA_OP_SUB && rs == 0) snprintf(buf, len, "NEG  r%u, r%u", rd, rt);
        else snprintf(buf, len, "%-4s r%u, r%u, r%u", names[op], rd, rs, rt);
        break;
    }
}

void pca_disasm_prog(const uint16_t *prog, int count)
{
    char b[64];
    for (int i = 0; i < count; i++) {
        pca_disasm(prog[i], b, sizeof b);
        printf("  0x%02X: %04X  %s\n", i, prog[i], b);
    }
}

/* ---- task JSON: tasks/spec.c:80-184 --------------------------------------- */

namespace {
const char *ws(const char *p)
{
    while (*p && isspace((unsigned char)*p)) p++;
    return p;
}

/* pointer just past `"key":` (first occurrence at or after p), or null */
const char *after_key(const char *p, const char *key)
{
    char pat[80];
    snprintf(pat, sizeof pat, "\"%s\"", key);
    const char *k = strstr(p, pat);
    if (!k) return nullptr;
    k = ws(k + strlen(pat));
    if (*k == ':') k++;
    return ws(k);
}

int int_list(const char *p, long *v, int maxn)
{
    int n = 0;
    p = ws(p);
    if (*p != '[') return 0;
    p++;
    while (n < maxn) {
        p = ws(p);
        if (*p == ']' || !*p) break;
        if (*p == ',') { p++; continue; }
        char *end;
        long x = strtol(p, &end, 10);
        if (end == p) break;
        v[n++] = x;
        p = end;
    }
    return n;
}
}  // namespace

int task_load(const char *path, task_spec_t *spec)
{
    memset(spec, 0, sizeof *spec);
    FILE *f = fopen(path, "rb");
    if (!f) { fprintf(stderr, "Cannot open task file: %s\n", path); return -1; }
    fseek(f, 0, SEEK_END);
    long size = ftell(f);
    fseek(f, 0, SEEK_SET);
    char *js = (char *)malloc((size_t)size + 1);
    if (!js) { fclose(f); return -1; }
    size_t got = fread(js, 1, (size_t)size, f);
    js[got] = 0;
    fclose(f);

    const char *p;
    if ((p = after_key(js, "name")) && *p == '"') {
        int i = 0;
        for (p++; *p && *p != '"' && i < 63; p++) spec->name[i++] = *p;
    }
    spec->max_cycles = (p = after_key(js, "max_cycles")) ? (uint64_t)strtol(p, nullptr, 10) : 1000;
    long v[MAX_IO_PORTS];
    if ((p = after_key(js, "input_ports"))) {
        spec->num_inputs = int_list(p, v, MAX_IO_PORTS);
        for (int i = 0; i < spec->num_inputs; i++) spec->input_ports[i] = (uint8_t)v[i];
    }
    if ((p = after_key(js, "output_ports"))) {
        spec->num_outputs = int_list(p, v, MAX_IO_PORTS);
        for (int i = 0; i < spec->num_outputs; i++) spec->output_ports[i] = (uint8_t)v[i];
    }
    if ((p = after_key(js, "tests"))) {
        p = ws(p);
        if (*p == '[') p++;
        /* at most MAX_TESTS tests are kept, as in tasks/spec.c:140 */
        while (spec->num_tests < MAX_TESTS) {
            p = ws(p);
            if (*p == ',') p = ws(p + 1);
            if (*p != '{') break;
            const char *obj = p;
            int depth = 0;
            do {
                if (*p == '{') depth++;
                else if (*p == '}') depth--;
                p++;
            } while (*p && depth > 0);
            test_case_t &tc = spec->tests[spec->num_tests];
            const char *q;
            if ((q = after_key(obj, "in"))) {
                int n = int_list(q, v, MAX_IO_PORTS);
                for (int i = 0; i < n; i++) tc.in[i] = (uint16_t)(v[i] & 0xFFFF);
            }
            if ((q = after_key(obj, "out"))) {
                int n = int_list(q, v, MAX_IO_PORTS);
                for (int i = 0; i < n; i++) tc.out[i] = (uint16_t)(v[i] & 0xFFFF);
            }
            spec->num_tests++;
        }
    }
    free(js);
    return 0;
}

/* tasks/spec.c:188-215 */
int task_evaluate(const task_spec_t *spec, const uint16_t *prog, int prog_len)
{
    int passed = 0;
    for (int t = 0; t < spec->num_tests; t++) {
        pca_vm_t vm;
        pca_init(&vm);
        pca_load(&vm, prog, (size_t)prog_len);
        for (int i = 0; i < spec->num_inputs; i++)
            vm.ports[spec->input_ports[i]] = spec->tests[t].in[i];
        pca_run(&vm, spec->max_cycles);
        if (vm.status != PCA_HALTED) continue;
        bool ok = true;
        for (int i = 0; i < spec->num_outputs && ok; i++)
            ok = vm.ports[spec->output_ports[i]] == spec->tests[t].out[i];
        passed += ok;
    }
    return passed;
}

/* tasks/spec.c:219-237 */
void task_print(const task_spec_t *spec)
{
    printf("Task: %s\n", spec->name);
    printf("  max_cycles: %llu\n", (unsigned long long)spec->max_cycles);
    printf("  inputs: ");
    for (int i = 0; i < spec->num_inputs; i++) printf("port%d ", spec->input_ports[i]);
    printf("\n  outputs: ");
    for (int i = 0; i < spec->num_outputs; i++) printf("port%d ", spec->output_ports[i]);
    printf("\n  tests: %d\n", spec->num_tests);
    for (int t = 0; t < spec->num_tests; t++) {
        printf("    [%d] in=(", t);
        for (int i = 0; i < spec->num_inputs; i++) printf("%s%u", i ? "," : "", spec->tests[t].in[i]);
        printf(") out=(");
        for (int i = 0; i < spec->num_outputs; i++) printf("%s%u", i ? "," : "", spec->tests[t].out[i]);
        printf(")\n");
    }
}

/* ---- search state: src/search_state.c:15-268 ------------------------------ */

int search_ctx_init(search_ctx_t *ctx, const task_spec_t *task)
{
    if (task->num_tests > MAX_TESTS || task->num_outputs != 1 ||
        task->num_inputs > PCA_NUM_REGS - 1)
        return -1;
    memset(ctx, 0, sizeof *ctx);
    ctx->task = *task;
    ctx->num_tests = (uint8_t)task->num_tests;
    ctx->num_inputs = (uint8_t)task->num_inputs;
    ctx->num_outputs = (uint8_t)task->num_outputs;
    for (int i = 0; i < task->num_inputs; i++) ctx->input_regs[i] = (uint8_t)(i + 1);
    ctx->output_port = task->output_ports[0];
    return 0;
}

void search_state_init_root(const search_ctx_t *ctx, search_state_t *s)
{
    memset(s, 0, sizeof *s);
    for (int t = 0; t < ctx->num_tests; t++)
        for (int i = 0; i < ctx->num_inputs; i++) s->regs[t][i + 1] = ctx->task.tests[t].in[i];
    for (int i = 0; i < ctx->num_inputs; i++) s->live |= (uint8_t)(1u << (i + 1));
}

int search_state_step(const search_ctx_t *ctx, const search_state_t *src, uint16_t insn,
                      search_state_t *dst)
{
    uint32_t op = PCA_INSN_OP(insn), rd = PCA_INSN_RD(insn);
    uint32_t rs = PCA_INSN_RS(insn), rt = PCA_INSN_RT(insn), imm = PCA_INSN_IMM(insn);
    bool alu = (op >= PCA_OP_ADD && op <= PCA_OP_ASR) || op == PCA_OP_LDI || op == PCA_OP_ADDI;
    if (!alu) return 0;
    *dst = *src;
    dst->depth = (uint8_t)(src->depth + 1);
    for (int t = 0; t < ctx->num_tests; t++) {
        uint16_t *r = dst->regs[t];
        uint32_t res, f;
        if (op == PCA_OP_DIV || op == PCA_OP_MOD) {
            /* division by zero on any test makes the instruction illegal */
            if (r[rt] == 0) return 0;
            res = op == PCA_OP_DIV ? (uint16_t)((int16_t)r[rs] / (int16_t)r[rt])
                                   : (uint16_t)((int16_t)r[rs] % (int16_t)r[rt]);
            f = pca_zn(res);
        } else {
            uint32_t a = op == PCA_OP_ADDI ? r[rd] : r[rs], b = r[rt];
            res = pca_alu(op, a, b, imm);
            f = pca_alu_flags(op, a, b, imm, res, dst->flags[t]);
        }
        r[rd] = (uint16_t)res;
        dst->flags[t] = (uint8_t)f;
        r[0] = 0;
    }
    if (rd != 0) dst->live = (uint8_t)(src->live | (1u << rd));
    return 1;
}

/* FNV-1a 64 over (lo, hi) of r0..r7 then flags, per test */
uint64_t search_state_oep_hash64(const search_ctx_t *ctx, const search_state_t *s)
{
    uint64_t h = 0xCBF29CE484222325ULL;
    auto mix = [&h](uint8_t b) { h = (h ^ b) * 0x00000100000001B3ULL; };
    for (int t = 0; t < ctx->num_tests; t++) {
        for (int r = 0; r < PCA_NUM_REGS; r++) {
            mix((uint8_t)(s->regs[t][r] & 0xFF));
            mix((uint8_t)(s->regs[t][r] >> 8));
        }
        mix(s->flags[t]);
    }
    return h;
}

uint64_t search_state_key_hash64(const search_ctx_t *ctx, const search_state_t *s)
{
    uint64_t h = search_state_oep_hash64(ctx, s);
    h = (h ^ s->live) * 0x00000100000001B3ULL;
    h = (h ^ s->depth) * 0x00000100000001B3ULL;
    return h;
}

uint8_t search_state_leaf_outputs(const search_ctx_t *ctx, const search_state_t *s)
{
    uint8_t out = 0;
    for (int r = 1; r < PCA_NUM_REGS; r++) {
        if (!((s->live >> r) & 1u)) continue;
        bool ok = true;
        for (int t = 0; t < ctx->num_tests && ok; t++) ok = s->regs[t][r] == ctx->task.tests[t].out[0];
        if (ok) out |= (uint8_t)(1u << r);
    }
    return out;
}

void search_state_serialize(const search_ctx_t *ctx, const search_state_t *s, uint32_t task_id,
                            uint16_t parent_action, uint8_t target_depth,
                            uint8_t can_finish_optimally, int8_t remaining_steps,
                            dataset_state_record_t *out)
{
    memset(out, 0, sizeof *out);
    out->state_hash = search_state_key_hash64(ctx, s);
    out->oep_hash = search_state_oep_hash64(ctx, s);
    out->task_id = task_id;
    out->parent_action = parent_action;
    out->depth = s->depth;
    out->budget_left = (uint8_t)(target_depth - s->depth);
    out->live = s->live;
    out->can_finish_optimally = can_finish_optimally;
    out->remaining_steps = remaining_steps;
    for (int t = 0; t < ctx->num_tests; t++) {
        memcpy(out->regs[t], s->regs[t], sizeof out->regs[t]);
        out->flags[t] = s->flags[t];
    }
}

int search_gen_candidates_branchless(uint16_t *out, int max, const search_state_t *s)
{
    return gen_candidates(s->live, out, max);
}

void search_state_dump(const search_ctx_t *ctx, const search_state_t *s, void *fpv)
{
    FILE *fp = (FILE *)fpv;
    fprintf(fp, "depth=%d live=0x%02X\n", s->depth, s->live);
    for (int t = 0; t < ctx->num_tests; t++) {
        fprintf(fp, "  test[%d] flags=%02X regs=[", t, s->flags[t]);
        for (int r = 0; r < PCA_NUM_REGS; r++) fprintf(fp, "%s%u", r ? "," : "", s->regs[t][r]);
        fprintf(fp, "]\n");
    }
}

int pcagb_num_candidates(uint8_t live) { return gen_tables().nc((live >> 1) & 127); }

}  // extern "C"
