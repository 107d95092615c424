"""Host half of libpcagb.so against the reference: the library loads and
exports every function include/pca_gb300.h declares; the libpca-compatible
search-state primitives reproduce the reference's outputs on recorded random
walks; task_evaluate and pca_disasm agree; the generator tables agree with
the oracle for all 128 liveness masks. No GPU calls."""
import ctypes
import hashlib
import os
import random
import re

import pytest

from conftest import REPO, load_golden, spec_from_json
from oracle import oracle as O
from pca_gb300.pcalib import EXPORTS, PCALib, SearchCtx, SearchState, load_library

LIBPCA = load_golden("ref_libpca.json")


def header_functions():
    text = open(os.path.join(REPO, "include", "pca_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = set(re.findall(r"\b([a-z_][a-z0-9_]*)\s*\(", text))
    return sorted(n for n in names if n not in {"if", "void", "sizeof"} and not n.startswith("on_"))


def test_exports_every_declared_symbol():
    lib = load_library()
    declared = header_functions()
    assert set(declared) == set(EXPORTS), set(declared) ^ set(EXPORTS)
    for name in declared:
        assert hasattr(lib, name), name


def test_struct_layouts():
    from pca_gb300.pcalib import TaskSpec
    # name, max_cycles, ports/counts, 32 tests, num_tests; padded to 8 bytes
    assert ctypes.sizeof(TaskSpec) == 1128
    assert ctypes.sizeof(SearchState) == 32 * 8 * 2 + 32 + 2
    assert SearchCtx.num_tests.offset == ctypes.sizeof(TaskSpec)


@pytest.mark.parametrize("walk", LIBPCA["walks"], ids=lambda w: w["task"]["name"])
def test_search_state_walks_match_reference(walk):
    L = PCALib()
    spec = spec_from_json(walk["task"])
    ctx = L.init_ctx(spec)
    s = L.init_root(ctx)
    for st in walk["steps"]:
        cands = L.gen_candidates(s)
        buf = (ctypes.c_uint16 * len(cands))(*cands)
        assert len(cands) == st["ncands"]
        assert hashlib.sha256(bytes(buf)).hexdigest()[:32] == st["cands_sha"]
        d = L.step(ctx, s, st["insn"])
        assert (d is not None) == bool(st["ok"])
        if d is None:
            break
        assert hashlib.sha256(bytes(d)).hexdigest()[:32] == st["state_sha"]
        assert str(L.oep_hash(ctx, d)) == st["oep"]
        assert str(L.key_hash(ctx, d)) == st["key"]
        assert L.leaf_check(ctx, d) == st["leaf"]
        s = d


def test_disasm_matches_reference():
    L = PCALib()
    for w, text in LIBPCA["disasm"].items():
        assert L.disasm(int(w)) == text


def test_generator_tables_match_oracle():
    L = PCALib()
    for m in range(128):
        live = m << 1
        s = SearchState()
        s.live = live
        assert L.gen_candidates(s) == O.gen_candidates(live)
        assert L.lib.pcagb_num_candidates(live) == len(O.gen_candidates(live))


def test_fixed_device_tables_hold_every_candidate():
    """The no-allocation solve keeps the candidates of all 128 liveness
    masks in fixed-size device arrays of kMaxTableCandidates entries: the
    generator must stay within that bound."""
    L = PCALib()
    total = sum(L.lib.pcagb_num_candidates(m << 1) for m in range(128))
    src = open(os.path.join(REPO, "pca_gb300", "csrc", "gen_tables.h")).read()
    bound = int(re.search(r"kMaxTableCandidates\s*=\s*(\d+)", src).group(1))
    assert total <= bound
    assert "pcagb::kMaxTableCandidates" in open(
        os.path.join(REPO, "pca_gb300", "csrc", "noalloc.cu")).read()


def test_step_matches_oracle_on_random_states():
    """Random register files and flags, every opcode word class."""
    L = PCALib()
    rng = random.Random(5)
    ol = O.lib()
    for trial in range(300):
        spec = spec_from_json({"name": "r", "max_cycles": 100, "input_ports": [0, 1],
                               "output_ports": [0],
                               "tests": [{"in": [rng.randrange(65536), rng.randrange(65536)],
                                          "out": [rng.randrange(65536)]} for _ in range(rng.randrange(1, 33))]})
        ctx = L.init_ctx(spec)
        s = SearchState()
        for t in range(32):
            for r in range(1, 8):
                s.regs[t][r] = rng.choice([0, 1, 0x8000, 0xFFFF, 0x7FFF, rng.randrange(65536)])
            s.flags[t] = rng.randrange(16)
        s.live = rng.randrange(256) & 0xFE
        s.depth = rng.randrange(5)
        insn = rng.randrange(65536)
        a = L.step(ctx, s, insn)
        b = SearchState()
        okb = ol.orc_step(ctypes.byref(ctx), ctypes.byref(s), insn, ctypes.byref(b))
        assert (a is not None) == bool(okb)
        if a is not None:
            assert bytes(a) == bytes(b)
            assert L.oep_hash(ctx, a) == ol.orc_oep_hash64(ctypes.byref(ctx), ctypes.byref(a))
            assert L.key_hash(ctx, a) == ol.orc_key_hash64(ctypes.byref(ctx), ctypes.byref(a))
            assert L.leaf_check(ctx, a) == ol.orc_leaf_outputs(ctypes.byref(ctx), ctypes.byref(a))


def test_task_load_and_evaluate(tmp_path):
    L = PCALib()
    fx = load_golden("ref_enumerate.json")
    for f in fx[:12]:
        p = tmp_path / "t.json"
        import json
        p.write_text(json.dumps(f["task"], indent=2))
        spec = L.load_task(str(p))
        ref = spec_from_json(f["task"])
        assert bytes(spec) == bytes(ref)
        for prog in f["programs"]:
            assert L.evaluate(spec, prog) == spec.num_tests
            bad = list(prog)
            bad[-2] ^= 1 << 8  # OUT from another register
            assert L.evaluate(spec, bad) <= spec.num_tests
    with pytest.raises(RuntimeError):
        L.load_task(str(tmp_path / "missing.json"))


def test_task_load_keeps_at_most_32_tests(tmp_path):
    import json
    L = PCALib()
    p = tmp_path / "big.json"
    p.write_text(json.dumps({"name": "big", "input_ports": [0], "output_ports": [0],
                             "tests": [{"in": [i], "out": [i]} for i in range(40)]}))
    spec = L.load_task(str(p))
    assert spec.num_tests == 32 and spec.max_cycles == 1000


def test_ctypes_mirrors_match_the_header(tmp_path):
    """Every ctypes mirror of a struct in include/pca_gb300.h has the C
    compiler's size and field offsets (a field appended to the header and
    not to the mirror, or the other way round, fails here)."""
    import shutil
    import subprocess
    from pca_gb300 import pcalib as P
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    mirrors = {"task_spec_t": P.TaskSpec, "search_state_t": P.SearchState,
               "search_ctx_t": P.SearchCtx, "pcagb_opts_t": P.SolveOpts,
               "pcagb_result_t": P.SolveResult, "pcagb_tuning_t": P.Tuning,
               "pcagb_server_config_t": P.ServerConfig, "pcagb_server_stats_t": P.ServerStats,
               "pcagb_level_view_t": P.LevelView, "pcagb_record_stats_t": P.RecordStats}
    lines = ['#include <stdio.h>', '#include "pca_gb300.h"', "int main(void) {"]
    for cname, cls in mirrors.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, *_ in cls._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)], check=True)
    got = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    want = []
    for cname, cls in mirrors.items():
        want.append(f"{cname} size {ctypes.sizeof(cls)}")
        for fname, *_ in cls._fields_:
            want.append(f"{cname} {fname} {getattr(cls, fname).offset}")
    assert [g for g in got if g] == want
