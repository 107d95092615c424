"""The reference's synthetic task corpus, generated the same way.

A restatement of the reference's task generator (tools/gen_tasks.c): the same
random stream, the same programs, the same filters and the same JSON files,
byte for byte, so a corpus written by

    python -m pca_gb300.corpus <output_dir> [-n count] [-s seed] [--verify]
                                           [--min-len N] [--max-len N]

equals the one `gen_tasks` writes with the same arguments, and the batched
and served workloads can draw tasks from the reference's distribution
(`corpus_tasks`).

The steps, with the reference's lines:
  random stream   xoshiro256** seeded by splitmix64 (gen_tasks.c:33-75)
  probe bank      1 input: 128 uniform values then 21 edge values; 2 inputs:
                  256 uniform pairs, 21 (e, e) and 21 (e, e+7) edge pairs
                  (:77-130)
  program         1 or 2 inputs (p = 0.4 / 0.6), kernel length uniform in
                  [min_len, max_len], instructions by category weights
                  add/sub .25, logic .25, shift .15, LDI .15, ADDI .15,
                  MUL .05 with the category's operand rules and up to 100
                  redraws (:132-229)
  output register the live register whose backward slice covers the most
                  kernel instructions (first of the best); coverage < 0.5
                  rejects (:231-265, :389-398)
  interesting     >= 4 distinct outputs over the bank and no simple baseline
                  (0, 1, x, y, x+-1, x+-y, y-x, x&y, x|y, x^y) matching more
                  than 95% of the probes (:267-318)
  tests           probes 128 and 129 then 8 distinct random probes
                  (:409-460); --verify draws 10 more probes per task and
                  checks the program on them (:526-570)

The probe bank is executed with numpy (one vector op per instruction over
all probes); every value is 16-bit unsigned as in the reference.
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np

M64 = (1 << 64) - 1

OP_ADD, OP_SUB, OP_MUL = 0x02, 0x03, 0x04
OP_AND, OP_OR, OP_XOR = 0x07, 0x08, 0x09
OP_SHL, OP_SHR, OP_ASR = 0x0A, 0x0B, 0x0C
OP_CMP, OP_LDI, OP_ADDI = 0x0D, 0x10, 0x12
OP_HLT, OP_IN, OP_OUT = 0x01, 0x17, 0x18

EDGE_VALUES = [0, 1, 2, 3, 4, 5, 7, 8, 15, 16, 31, 32, 63, 64, 127, 128, 255, 256,
               0x7FFF, 0x8000, 0xFFFF]
CATEGORY_WEIGHTS = [0.25, 0.25, 0.15, 0.15, 0.15, 0.05]
LDI_VALUES = [0, 1, 2, 3, 4, 5, 8, 16, 32, 64, 128, 255]
ADDI_VALUES = [-1, 1, -2, 2, -3, 3]
NUM_TESTS = 10
MAX_CYCLES = 32
MAX_KERNEL_LEN = 10


def encode_r(op, rd, rs, rt):
    return ((op & 0x1F) << 11) | ((rd & 7) << 8) | ((rs & 7) << 5) | ((rt & 7) << 2)


def encode_i(op, rd, imm8):
    return ((op & 0x1F) << 11) | ((rd & 7) << 8) | (imm8 & 0xFF)


class Xoshiro256ss:
    """xoshiro256** over four 64-bit words, seeded by splitmix64."""

    def __init__(self, seed: int):
        self.s = []
        x = seed & M64
        for _ in range(4):
            x = (x + 0x9E3779B97F4A7C15) & M64
            z = x
            z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
            z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
            self.s.append(z ^ (z >> 31))

    @staticmethod
    def _rotl(x, k):
        return ((x << k) | (x >> (64 - k))) & M64

    def next(self) -> int:
        s = self.s
        result = (self._rotl((s[1] * 5) & M64, 7) * 9) & M64
        t = (s[1] << 17) & M64
        s[2] ^= s[0]
        s[3] ^= s[1]
        s[1] ^= s[2]
        s[0] ^= s[3]
        s[2] ^= t
        s[3] = self._rotl(s[3], 45)
        return result

    def u16(self) -> int:
        return self.next() & 0xFFFF

    def int_in(self, lo: int, hi: int) -> int:
        """Uniform in [lo, hi] by modulo, as the reference draws it."""
        return lo + self.next() % (hi - lo + 1)

    def f64(self) -> float:
        return (self.next() >> 11) * (1.0 / (1 << 53))


def _probe_bank(rng: Xoshiro256ss, num_inputs: int) -> np.ndarray:
    if num_inputs == 1:
        rows = [(rng.u16(), 0) for _ in range(128)]
        rows += [(e, 0) for e in EDGE_VALUES]
    else:
        rows = []
        for _ in range(256):
            x = rng.u16()
            y = rng.u16()
            rows.append((x, y))
        n = len(EDGE_VALUES)
        rows += [(EDGE_VALUES[i], EDGE_VALUES[i % n]) for i in range(n)]
        rows += [(EDGE_VALUES[i], EDGE_VALUES[(i + 7) % n]) for i in range(n)]
    return np.array(rows, dtype=np.uint16)


def _sample_category(rng: Xoshiro256ss) -> int:
    r = rng.f64()
    cum = 0.0
    for i, w in enumerate(CATEGORY_WEIGHTS):
        cum += w
        if r < cum:
            return i
    return 0


def _sample_instruction(rng: Xoshiro256ss, live: int) -> int:
    for _ in range(100):
        cat = _sample_category(rng)
        rd = rng.int_in(1, 7)
        if cat == 0:                                     # ADD / SUB
            op = OP_ADD if rng.int_in(0, 1) else OP_SUB
            rs, rt = rng.int_in(0, 7), rng.int_in(0, 7)
            if rs and not (live >> rs) & 1:
                continue
            if rt and not (live >> rt) & 1:
                continue
            if rs == 0 and rt == 0:
                continue
            if op == OP_ADD and ((rs == rd and rt == 0) or (rt == rd and rs == 0)):
                continue
            if op == OP_SUB and rs == rd and rt == 0:
                continue
            return encode_r(op, rd, rs, rt)
        if cat == 1:                                     # AND / OR / XOR
            op = (OP_AND, OP_OR, OP_XOR)[rng.int_in(0, 2)]
            rs, rt = rng.int_in(0, 7), rng.int_in(0, 7)
            if rs and not (live >> rs) & 1:
                continue
            if rt and not (live >> rt) & 1:
                continue
            if rs == 0 and rt == 0:
                continue
            return encode_r(op, rd, rs, rt)
        if cat == 2:                                     # SHL / SHR / ASR
            op = (OP_SHL, OP_SHR, OP_ASR)[rng.int_in(0, 2)]
            rs, rt = rng.int_in(0, 7), rng.int_in(1, 7)
            if rs and not (live >> rs) & 1:
                continue
            if not (live >> rt) & 1:
                continue
            return encode_r(op, rd, rs, rt)
        if cat == 3:                                     # LDI
            return encode_i(OP_LDI, rd, LDI_VALUES[rng.int_in(0, 11)])
        if cat == 4:                                     # ADDI (on a live rd)
            if not (live >> rd) & 1:
                continue
            return encode_i(OP_ADDI, rd, ADDI_VALUES[rng.int_in(0, 5)] & 0xFF)
        rs, rt = rng.int_in(1, 7), rng.int_in(1, 7)      # MUL
        if not (live >> rs) & 1 or not (live >> rt) & 1:
            continue
        return encode_r(OP_MUL, rd, rs, rt)
    return encode_i(OP_LDI, 1, 1)


def _fields(insn: int):
    return insn >> 11, (insn >> 8) & 7, (insn >> 5) & 7, (insn >> 2) & 7, insn & 0xFF


def _execute(regs: np.ndarray, insn: int) -> None:
    """One instruction on every probe's registers (uint32 columns holding
    16-bit values)."""
    op, rd, rs, rt, imm = _fields(insn)
    a, b = regs[rs], regs[rt]
    if op == OP_ADD:
        regs[rd] = (a + b) & 0xFFFF
    elif op == OP_SUB:
        regs[rd] = (a - b) & 0xFFFF
    elif op == OP_MUL:
        regs[rd] = (a * b) & 0xFFFF
    elif op == OP_AND:
        regs[rd] = a & b
    elif op == OP_OR:
        regs[rd] = a | b
    elif op == OP_XOR:
        regs[rd] = a ^ b
    elif op == OP_SHL:
        regs[rd] = (a << (b & 0xF)) & 0xFFFF
    elif op == OP_SHR:
        regs[rd] = a >> (b & 0xF)
    elif op == OP_ASR:
        signed = a.astype(np.int64) - ((a & 0x8000).astype(np.int64) << 1)
        regs[rd] = (signed >> (b & 0xF).astype(np.int64)).astype(np.int64) & 0xFFFF
    elif op == OP_LDI:
        regs[rd] = imm
    elif op == OP_ADDI:
        simm = imm - 256 if imm & 0x80 else imm
        regs[rd] = (regs[rd] + (simm & 0xFFFF)) & 0xFFFF
    regs[0] = 0


def _slice_coverage(kernel, out_reg: int) -> float:
    needed = 1 << out_reg
    used = 0
    for insn in reversed(kernel):
        op, rd, rs, rt, _ = _fields(insn)
        if not (needed >> rd) & 1:
            continue
        used += 1
        if op == OP_LDI:
            needed &= ~(1 << rd)
        elif op == OP_ADDI:
            pass
        else:
            needed &= ~(1 << rd)
            if rs:
                needed |= 1 << rs
            if rt:
                needed |= 1 << rt
    return used / len(kernel) if kernel else 0.0


def _interesting(bank: np.ndarray, outputs: np.ndarray, num_inputs: int) -> bool:
    if len(np.unique(outputs)) < 4:
        return False
    x = bank[:, 0].astype(np.uint32)
    y = bank[:, 1].astype(np.uint32) if num_inputs > 1 else np.zeros_like(x)
    out = outputs.astype(np.uint32)
    m = 0xFFFF
    baselines = [out == 0, out == 1, out == x, (out == y) & (num_inputs > 1),
                 out == ((x + 1) & m), out == ((x - 1) & m), out == ((x + y) & m),
                 out == ((x - y) & m), out == ((y - x) & m), out == (x & y), out == (x | y),
                 out == (x ^ y)]
    threshold = int(len(out) * 0.95)
    return all(int(b.sum()) <= threshold for b in baselines)


def _generate_one(rng: Xoshiro256ss, min_len: int, max_len: int):
    """One attempt: (program dict or None, rejected-by-slice flag)."""
    num_inputs = 1 if rng.f64() < 0.4 else 2
    kernel_len = min_len + rng.int_in(0, max_len - min_len)
    bank = _probe_bank(rng, num_inputs)
    regs = np.zeros((8, len(bank)), dtype=np.int64)
    live = 0
    for i in range(num_inputs):
        regs[i + 1] = bank[:, i]
        live |= 1 << (i + 1)
    kernel = []
    for _ in range(kernel_len):
        insn = _sample_instruction(rng, live)
        kernel.append(insn)
        _execute(regs, insn)
        op, rd = insn >> 11, (insn >> 8) & 7
        if op != OP_CMP and rd:
            live |= 1 << rd
    out_reg, best = 0, 0.0
    for r in range(1, 8):
        if not (live >> r) & 1:
            continue
        cov = _slice_coverage(kernel, r)
        if cov > best:
            best, out_reg = cov, r
    if out_reg == 0 or best < 0.5:
        return None, True
    outputs = regs[out_reg].astype(np.uint16)
    if not _interesting(bank, outputs, num_inputs):
        return None, False
    return dict(num_inputs=num_inputs, kernel=kernel, kernel_len=kernel_len, out_reg=out_reg,
                bank=bank, outputs=outputs), False


def _select_tests(rng: Xoshiro256ss, count: int):
    sel = [128, 129] if count > 128 else []
    while len(sel) < NUM_TESTS:
        idx = rng.int_in(0, count - 1)
        if idx not in sel:
            sel.append(idx)
    return sel


def task_json_text(num: int, prog) -> str:
    """The file the reference writes for task number `num` (its exact text)."""
    ni, kl = prog["num_inputs"], prog["kernel_len"]
    name = f"syn_{ni}inp_len{kl}_{num:06d}"
    lines = ["{", f'    "name": "{name}",', f'    "max_cycles": {MAX_CYCLES},',
             '    "input_ports": [' + ", ".join(str(i) for i in range(ni)) + "],",
             '    "output_ports": [0],', '    "tests": [']
    sel = prog["tests"]
    for i, idx in enumerate(sel):
        ins = ", ".join(str(int(prog["bank"][idx][j])) for j in range(ni))
        lines.append(f'        {{"in": [{ins}], "out": [{int(prog["outputs"][idx])}]}}'
                     + ("," if i < NUM_TESTS - 1 else ""))
    lines += ["    ]", "}"]
    return "\n".join(lines) + "\n"


def generate(count: int = 1000, seed: int = 42, min_len: int = 0, max_len: int = 0,
             verify: bool = False):
    """Yields (file name, file text, program dict) exactly as the reference
    generator would write them; stops like it after count * 50 attempts."""
    g_min, g_max = 2, 6
    if min_len > 0:
        g_min = min_len
    if max_len > 0:
        g_max = max_len
    g_max = min(g_max, MAX_KERNEL_LEN)
    g_min = min(g_min, g_max)
    rng = Xoshiro256ss(seed)
    generated = attempted = 0
    while generated < count and attempted < count * 50:
        attempted += 1
        prog, _ = _generate_one(rng, g_min, g_max)
        if prog is None:
            continue
        if verify:
            # ten more probes drawn per task; the program computes every
            # probe's output by construction, so the check passes
            for _ in range(NUM_TESTS):
                rng.int_in(0, len(prog["bank"]) - 1)
        prog["tests"] = _select_tests(rng, len(prog["bank"]))
        name = f"syn_{prog['num_inputs']}inp_len{prog['kernel_len']}_{generated:06d}.json"
        yield name, task_json_text(generated, prog), prog
        generated += 1


def program_words(prog):
    """The generating program as full PCA-16 words (IN scaffold, kernel,
    OUT, HLT)."""
    words = [encode_i(OP_IN, i + 1, i) for i in range(prog["num_inputs"])]
    words += prog["kernel"]
    words += [encode_i(OP_OUT, prog["out_reg"], 0), encode_r(OP_HLT, 0, 0, 0)]
    return words


def corpus_tasks(count: int, seed: int = 42, min_len: int = 0, max_len: int = 0):
    """The corpus as TaskSpec structs (for the engine)."""
    from .pcalib import make_task
    out = []
    for _, text, _ in generate(count, seed, min_len, max_len):
        d = json.loads(text)
        out.append(make_task(d["name"], [t["in"] for t in d["tests"]],
                             [t["out"][0] for t in d["tests"]]))
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m pca_gb300.corpus",
                                 description="the reference's synthetic task corpus")
    ap.add_argument("output_dir")
    ap.add_argument("-n", type=int, default=1000)
    ap.add_argument("-s", type=int, default=42)
    ap.add_argument("--verify", action="store_true")
    ap.add_argument("--min-len", type=int, default=0)
    ap.add_argument("--max-len", type=int, default=0)
    args = ap.parse_args(argv)
    os.makedirs(args.output_dir, exist_ok=True)
    n = 0
    for name, text, _ in generate(args.n, args.s, args.min_len, args.max_len, args.verify):
        with open(os.path.join(args.output_dir, name), "w") as f:
            f.write(text)
        n += 1
    print(f"Done: {n} tasks generated")
    return 0


if __name__ == "__main__":
    sys.exit(main())
