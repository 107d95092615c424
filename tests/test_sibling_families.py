"""The insert kernel leaves out candidates whose child is an earlier
sibling's state, by fixed families of the generator's list (copies of a
register with its Z/N flags, zero with Z, zero with Z and C; engine.cu
uploads them as bit 31 of the device micro-ops). The families are checked
here on the host, through the product's own step function: every member of
a family reaches the same registers and flags as its first member, from
random states of every liveness mask, and the first member is the earliest
in the generator's order. (On the GPU the same rule is covered by the
survivor-count and program parity tests, which would change if a child of
a different state were left out.)"""
import random

from pca_gb300.pcalib import PCALib, SearchState

ADD, SUB, AND, OR, XOR, SHL, SHR, ASR = 0x02, 0x03, 0x07, 0x08, 0x09, 0x0A, 0x0B, 0x0C


def fields(w):
    return (w >> 11) & 31, (w >> 8) & 7, (w >> 5) & 7, (w >> 2) & 7


def family(w):
    op, rd, a, b = fields(w)
    if op in (ADD, OR, XOR) and a == 0 and b >= 1:
        return ("copy", rd, b)
    if op in (AND, OR) and a == b and a >= 1:
        return ("copy", rd, a)
    if op in (AND, SHL, SHR, ASR) and a == 0 and b >= 1:
        return ("zero", rd)
    if op == XOR and a == b and a >= 1:
        return ("zero", rd)
    if op == SUB and a == b and a >= 1:
        return ("zero_c", rd)
    return None


def test_op_codes_match_the_isa():
    import os
    hdr = open(os.path.join(os.path.dirname(__file__), "..", "pca_gb300", "csrc", "pca_isa.h")).read()
    for name, code in (("ADD", ADD), ("SUB", SUB), ("AND", AND), ("OR", OR), ("XOR", XOR),
                       ("SHL", SHL), ("SHR", SHR), ("ASR", ASR)):
        assert f"PCA_OP_{name} = 0x{code:02X}" in hdr


def test_family_members_reach_the_first_members_state():
    lib = PCALib()
    from pca_gb300.taskgen import synthetic_task
    task = synthetic_task(3, 2)[0]
    ctx = lib.init_ctx(task)
    rng = random.Random(5)
    checked = 0
    for mask in range(128):
        live = (mask << 1) | 2
        st = SearchState()
        st.live = live
        cands = lib.gen_candidates(st)
        groups = {}
        for i, w in enumerate(cands):
            k = family(w)
            if k is not None:
                groups.setdefault(k, []).append(i)
        for _ in range(3):
            src = SearchState()
            src.live = live
            for t in range(task.num_tests):
                for r in range(1, 8):
                    src.regs[t][r] = rng.getrandbits(16) if (live >> r) & 1 else 0
                src.flags[t] = rng.getrandbits(4)
            for k, members in groups.items():
                ref = lib.step(ctx, src, cands[members[0]])
                assert ref is not None
                for i in members[1:]:
                    assert i > members[0]
                    got = lib.step(ctx, src, cands[i])
                    for t in range(task.num_tests):
                        assert list(got.regs[t]) == list(ref.regs[t]), (hex(cands[i]), k)
                        assert got.flags[t] == ref.flags[t], (hex(cands[i]), k)
                    assert got.live == ref.live
                    checked += 1
    assert checked > 1000
