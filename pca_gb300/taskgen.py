"""Seeded synthetic task generators for the benchmark workloads.

No public suite is involved: every workload is generated from a seed.

  negate_task      r1 = -x mod 2^16; 16 tests: 11 uniform 16-bit values plus
                   0, 1, 0xFFFF, 0x7FFF, 0x8000.
  is_power2_task   r1 = 1 if x is a power of two else 0; 32 tests: 12 powers
                   of two below 2^15, 0, 0x8000, 18 uniform non-powers.
  random_program / synthetic_task
                   a random branchless program (ops uniform over ADD SUB MUL
                   AND OR XOR SHL SHR ASR LDI ADDI, registers uniform r1..r7,
                   immediates half 0..15, half uniform 16-bit), run on 16..32
                   tests of 1..2 uniform 16-bit inputs; the output is the last
                   written register. Programs with 16-bit immediates are not
                   encodable, so a task may need more than its source length.
  synthetic_batch  1,000 such tasks of source length 3..8 (batched workload).
  poisson_stream   arrival times at rate 50/s with source length mix
                   4:30%, 5:30%, 6:25%, 7:10%, 8:5% (served workload).
  deep_tasks       200 tasks of source length 8..10 (value-ordered workload).
"""
from __future__ import annotations

import random

from .pcalib import make_task

BRANCHLESS_OPS = ["ADD", "SUB", "MUL", "AND", "OR", "XOR", "SHL", "SHR", "ASR", "LDI", "ADDI"]


def negate_task(seed: int = 1):
    rng = random.Random(seed)
    xs = [rng.randrange(1 << 16) for _ in range(11)] + [0, 1, 0xFFFF, 0x7FFF, 0x8000]
    return make_task("negate", [[x] for x in xs], [(-x) & 0xFFFF for x in xs])


def is_power2_task(seed: int = 1):
    rng = random.Random(seed)
    pows = rng.sample([1 << k for k in range(15)], 12)
    non = []
    while len(non) < 18:
        x = rng.randrange(1 << 16)
        if x and (x & (x - 1)) and x not in non:
            non.append(x)
    xs = pows + [0, 0x8000] + non
    rng.shuffle(xs)
    return make_task("is_power2", [[x] for x in xs],
                     [1 if x and not (x & (x - 1)) else 0 for x in xs])


def _imm(rng: random.Random) -> int:
    return rng.randrange(16) if rng.random() < 0.5 else rng.randrange(1 << 16)


def random_program(rng: random.Random, length: int):
    prog = []
    for _ in range(length):
        op = rng.choice(BRANCHLESS_OPS)
        rd = rng.randrange(1, 8)
        if op in ("LDI", "ADDI"):
            prog.append((op, rd, 0, 0, _imm(rng)))
        else:
            prog.append((op, rd, rng.randrange(1, 8), rng.randrange(1, 8), 0))
    return prog


def run_program(prog, inputs):
    r = [0] * 8
    for i, v in enumerate(inputs):
        r[i + 1] = v & 0xFFFF
    for op, rd, rs, rt, imm in prog:
        a, b = r[rs], r[rt]
        if op == "ADD":
            v = a + b
        elif op == "SUB":
            v = a - b
        elif op == "MUL":
            v = a * b
        elif op == "AND":
            v = a & b
        elif op == "OR":
            v = a | b
        elif op == "XOR":
            v = a ^ b
        elif op == "SHL":
            v = a << (b & 15)
        elif op == "SHR":
            v = a >> (b & 15)
        elif op == "ASR":
            sa = a - 0x10000 if a & 0x8000 else a
            v = sa >> (b & 15)
        elif op == "LDI":
            v = imm
        else:  # ADDI
            v = r[rd] + imm
        r[rd] = v & 0xFFFF
        r[0] = 0
    return r


def synthetic_task(seed: int, length: int, name: str | None = None):
    rng = random.Random(seed)
    n_in = rng.randrange(1, 3)
    n_tests = rng.randrange(16, 33)
    prog = random_program(rng, length)
    out_reg = prog[-1][1]
    ins = [[rng.randrange(1 << 16) for _ in range(n_in)] for _ in range(n_tests)]
    outs = [run_program(prog, row)[out_reg] for row in ins]
    task = make_task(name or f"syn_{seed}_len{length}", ins, outs)
    return task, prog


def synthetic_batch(n: int = 1000, seed: int = 7, lengths=(3, 8)):
    rng = random.Random(seed)
    out = []
    for i in range(n):
        length = rng.randrange(lengths[0], lengths[1] + 1)
        out.append(synthetic_task(rng.randrange(1 << 62), length, f"syn{i:04d}_len{length}")[0])
    return out


def poisson_stream(n: int = 200, rate: float = 50.0, seed: int = 11):
    """[(arrival_seconds, task)] with the served workload's depth mix."""
    rng = random.Random(seed)
    mix = [(4, 0.30), (5, 0.30), (6, 0.25), (7, 0.10), (8, 0.05)]
    t = 0.0
    out = []
    for i in range(n):
        t += rng.expovariate(rate)
        u, acc, length = rng.random(), 0.0, 8
        for L, p in mix:
            acc += p
            if u < acc:
                length = L
                break
        out.append((t, synthetic_task(rng.randrange(1 << 62), length, f"req{i:04d}_len{length}")[0]))
    return out


def deep_tasks(n: int = 200, seed: int = 13):
    return synthetic_batch(n, seed, lengths=(8, 10))
