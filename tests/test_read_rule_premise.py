"""The suffix kernels scan only last instructions that read the register the
instruction before wrote (and skip middles that overwrite an unread write):
at the optimal depth no instruction of a solving program is unread, since
dropping it would leave a shorter solving program. Checked here on the
oracle's full canonical sets at the optimal depth (every solving program,
no pruning; 49 fixture tasks pinned to the reference): in every program each
kernel instruction's write is read by a later instruction (or is the one the
OUT reads) before it is overwritten."""
from conftest import load_golden

MODES = [m for m in load_golden("oracle_modes.json") if "full" in m]
ENUM = load_golden("ref_enumerate.json")
LDI, ADDI, OUT = 0x10, 0x12, 0x18


def decode(w):
    return (w >> 11) & 31, (w >> 8) & 7, (w >> 5) & 7, (w >> 2) & 7


def reads(w):
    op, rd, a, b = decode(w)
    if op == LDI:
        return set()
    if op == ADDI:
        return {rd}
    return {a, b}


def test_no_unread_write_at_the_optimal_depth():
    checked = 0
    for m in MODES:
        fx = ENUM[m["index"]]
        n_in = len(fx["task"]["input_ports"])
        for prog in m["full"]["programs"]:
            kernel = prog[n_in:-2]
            out_op, out_reg, _, _ = decode(prog[-2])
            assert out_op == OUT
            if not kernel:
                continue
            # the OUT reads the last write
            assert decode(kernel[-1])[1] == out_reg, prog
            for i, w in enumerate(kernel[:-1]):
                r = decode(w)[1]
                used = False
                for u in kernel[i + 1:]:
                    if r in reads(u):
                        used = True
                        break
                    if decode(u)[1] == r:
                        break
                assert used, (prog, i)
            checked += 1
    assert checked > 100
