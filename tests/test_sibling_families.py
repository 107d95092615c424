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


LDI, ADDI = 0x10, 0x12


def reads(w, r):
    op, rd, a, b = fields(w)
    if op == LDI:
        return False
    if op == ADDI:
        return rd == r
    return a == r or b == r


def random_state(live, T, rng):
    s = SearchState()
    s.live = live
    for t in range(T):
        for r in range(1, 8):
            s.regs[t][r] = rng.getrandbits(16) if (live >> r) & 1 else 0
        s.flags[t] = rng.getrandbits(4)
    return s


def same(a, b, T):
    return all(list(a.regs[t]) == list(b.regs[t]) and a.flags[t] == b.flags[t] for t in range(T)) \
        and a.live == b.live


def test_ldi_swap_and_dead_write_reach_the_same_state():
    """The insert kernel's two ordering rules, on the host: an LDI of
    register y and an instruction x that neither reads nor writes y give the
    same state in either order; two writes z, z' of register w followed by an
    instruction that is not an LDI and overwrites w without reading it give
    the same state."""
    lib = PCALib()
    from pca_gb300.taskgen import synthetic_task
    task = synthetic_task(3, 2)[0]
    ctx = lib.init_ctx(task)
    T = task.num_tests
    rng = random.Random(9)
    swaps = dead = 0
    for mask in range(0, 128, 3):
        live = (mask << 1) | 2
        cands = lib.gen_candidates(random_state(live, T, rng))
        ldis = [w for w in cands if fields(w)[0] == LDI]
        others = [w for w in cands if fields(w)[0] != LDI]
        for _ in range(40):
            src = random_state(live, T, rng)
            y = rng.choice(ldis)
            ry = fields(y)[1]
            x = rng.choice(others)
            if fields(x)[1] == ry or reads(x, ry) or fields(x)[0] == ADDI:
                continue
            a = lib.step(ctx, lib.step(ctx, src, y), x)
            b = lib.step(ctx, lib.step(ctx, src, x), y)
            if a is None or b is None:
                continue
            assert same(a, b, T), (hex(y), hex(x))
            swaps += 1
        for _ in range(40):
            src = random_state(live, T, rng)
            z1, z2 = rng.choice(cands), rng.choice(cands)
            w = fields(z1)[1]
            if fields(z2)[1] != w:
                continue
            s1, s2 = lib.step(ctx, src, z1), lib.step(ctx, src, z2)
            if s1 is None or s2 is None:
                continue
            follow = [u for u in lib.gen_candidates(s1)
                      if fields(u)[1] == w and fields(u)[0] != LDI and not reads(u, w)]
            if not follow:
                continue
            u = rng.choice(follow)
            a, b = lib.step(ctx, s1, u), lib.step(ctx, s2, u)
            assert a is not None and b is not None and same(a, b, T), (hex(z1), hex(z2), hex(u))
            dead += 1
    assert swaps > 200 and dead > 200
