"""The native library on the host: it loads, exports every entry point that
include/bbscite_gb300.h declares, and its host-side tree helpers and input
parser reproduce the reference's known answers.  No GPU is needed."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from bbscite_gb300 import data as D

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    with open(os.path.join(ROOT, "include", "bbscite_gb300.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"BBS_API [^;]*?\b(bbs_\w+)\(", text)))


def test_exports_every_declared_symbol(native):
    syms = declared_symbols()
    assert len(syms) >= 25
    L = C.CDLL(native.LIB_PATH)
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing


def test_defaults_match_reference_parameters(native):
    p = native.default_params()
    # src/Parameters.hpp:39-45
    assert p.alpha_mean == pytest.approx(6.04e-5)
    assert p.beta_mean == pytest.approx(0.4309)
    assert p.beta_sd == pytest.approx(0.1)
    assert (p.prob_beta_change, p.prob_prune_n_reattach, p.prob_swap_nodes,
            p.prob_swap_subtrees) == pytest.approx((0.0, 0.55, 0.4, 0.05))
    assert p.beta_jump_scaling_chi == 10.0 and p.gamma == 1.0


def test_host_tree_helpers_kat(native, kat):
    k = kat["pruefer_code_to_parent_vector"]
    assert native.pruefer_to_parent(k["code"]).tolist() == k["expected"]
    k = kat["parent_vector_to_matrix"]
    am, dm = native.parent_to_matrix(k["parent_vector"])
    assert [int(r[0]) for r in am] == [int(s, 2) for s in k["am"]]
    assert [int(r[0]) for r in dm] == [int(s, 2) for s in k["dm"]]
    assert (native.dm_to_am(dm) == am).all()
    assert native.matrix_to_parent(dm).tolist() == k["parent_vector"]
    pv = kat["to_graphviz"]["parent_vector"]
    assert native.to_graphviz(pv) == kat["to_graphviz"]["expected"]
    assert native.to_newick(pv) == kat["to_newick"]["expected"]


def test_host_helpers_match_oracle(native, orc):
    rng = np.random.default_rng(5)
    for G in (2, 5, 31, 63, 64, 95, 127, 128, 200, 255):
        code = rng.integers(0, G + 1, size=G - 1)
        pv = native.pruefer_to_parent(code)
        assert (pv == orc.pruefer_to_parent(code)).all()
        am, dm = native.parent_to_matrix(pv)
        oam, odm = orc.parent_to_matrix(pv)
        assert (am == oam).all() and (dm == odm).all()
        assert (native.matrix_to_parent(dm) == orc.parent_vector(dm)).all()


def test_random_parents_are_valid_trees(native):
    P = native.random_parents(123, 95, 64)
    assert P.shape == (64, 96)
    for pv in P:
        native.parent_to_matrix(pv)  # raises on an invalid tree
    assert not (P[0] == P[1]).all()
    assert (native.random_parents(123, 95, 64) == P).all()


def test_invalid_parent_vectors_are_rejected(native):
    with pytest.raises(native.BbsError) as e:
        native.parent_to_matrix([1, 0, 3, 3])  # cycle 0 -> 1 -> 0
    assert e.value.code == native.BBS_ERR_INPUT
    with pytest.raises(native.BbsError):
        native.parent_to_matrix([3, 0, 1, 2])  # root not its own parent
    with pytest.raises(native.BbsError):
        native.parent_to_matrix([9, 3, 3, 3])  # out of range


def test_read_csv_matches_generator(native, tmp_path):
    m, _, _ = D.generate_dataset(3, 40, 70, 1e-2, 0.2, 0.1, 0.05)
    path = str(tmp_path / "in.csv")
    D.write_csv(m, path)
    mut, known, nc, ng = native.read_csv(path)
    assert (nc, ng) == (70, 40)
    em, ek = D.matrix_to_bits(m)
    assert (mut == em).all() and (known == ek).all()


@pytest.mark.parametrize("text,err", [
    ("0 1 2\n0 1\n", "Inconsistent rows"),
    ("0 1 x\n", "Illegal character"),
    ("", "Empty input file"),
])
def test_read_csv_errors(native, tmp_path, text, err):
    path = tmp_path / "bad.csv"
    path.write_text(text)
    with pytest.raises(native.BbsError) as e:
        native.read_csv(str(path))
    assert err in str(e.value)


def test_read_csv_size_cap(native, tmp_path):
    path = tmp_path / "wide.csv"
    path.write_text("\n".join(["0 1"] * 256) + "\n")
    with pytest.raises(native.BbsError) as e:
        native.read_csv(str(path))
    assert e.value.code == native.BBS_ERR_SIZE


def test_create_without_gpu_fails_cleanly(native):
    from conftest import has_gpu
    if has_gpu():
        pytest.skip("a GPU is present")
    mut = np.zeros((4, 1), dtype=np.uint64)
    with pytest.raises(native.BbsError) as e:
        native.Context(mut, mut, 4, 10)
    assert e.value.code == native.BBS_ERR_CUDA


def test_create_validates_arguments(native):
    mut = np.zeros((4, 1), dtype=np.uint64)
    with pytest.raises(native.BbsError) as e:
        native.Context(mut, mut, 4, 1)  # fewer than 2 genes
    assert e.value.code == native.BBS_ERR_SIZE
    p = native.default_params(prob_beta_change=0.0, prob_prune_n_reattach=0.0,
                              prob_swap_nodes=0.0, prob_swap_subtrees=0.0)
    with pytest.raises(native.BbsError) as e:
        native.Context(mut, mut, 4, 10, p)
    assert "sum of the move type probabilities is zero" in str(e.value)


def test_shared_memory_layout_of_every_launch_shape(tmp_path):
    """tests/cpp/layout_probe.cu walks the chain kernels' shared-memory
    layout (the slot and table sizes and the per-warp pieces the kernels
    address) over every node count, cells per lane, warps per chain and
    chains per block that the launchers accept, with and without inherited
    counts: every piece lies inside its slot, the pieces are disjoint and
    aligned, and the increment tables fit after the slots."""
    import subprocess
    from bbscite_gb300 import build as B
    exe = str(tmp_path / "layout_probe")
    subprocess.run([B.nvcc(), *B.ARCH, "-std=c++17", "-I" + B.INCLUDE,
                    "-I" + B.CSRC,
                    os.path.join(ROOT, "tests", "cpp", "layout_probe.cu"),
                    "-o", exe], check=True, capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout
    assert r.stdout.startswith("layout ok "), r.stdout
    assert int(r.stdout.split()[2]) == 255 * 4 * 2 * 2 * 11


def _ctype_of(decl: str):
    """The ctypes type a C parameter or return declaration passes as."""
    d = " ".join(decl.replace("const ", "").split())
    if "*" in d:
        return C.c_char_p if d.startswith("char") else C.c_void_p
    base = d.split()[0] if d else "void"
    return {"void": None, "int": C.c_int, "int32_t": C.c_int32,
            "uint32_t": C.c_uint32, "uint64_t": C.c_uint64,
            "float": C.c_float, "size_t": C.c_size_t}[base]


def test_binding_signatures_match_the_header(native):
    """Every entry point the Python binding declares passes the argument
    count and scalar widths that include/bbscite_gb300.h declares (a drift
    between the two would pass wrong values silently through ctypes)."""
    with open(os.path.join(ROOT, "include", "bbscite_gb300.h")) as f:
        text = re.sub(r"/\*.*?\*/|//[^\n]*", "", f.read(), flags=re.S)
    decls = {}
    for ret, name, params in re.findall(
            r"BBS_API\s+([^;()]*?)\b(bbs_\w+)\s*\(([^)]*)\)\s*;", text):
        ps = [p.strip() for p in params.split(",")]
        if ps == ["void"]:
            ps = []
        # the parameter's type is the declaration less its name
        types = [re.sub(r"\b\w+\s*$", "", p) if not p.endswith("*") else p
                 for p in ps]
        decls[name] = (_ctype_of(ret.strip()), [_ctype_of(t) for t in types])
    L = native.lib()
    bound = [n for n in decls if getattr(L, n).argtypes is not None]
    assert len(bound) >= 40
    for name in bound:
        fn = getattr(L, name)
        want_ret, want_args = decls[name]
        # any pointer passes as a pointer; only returned strings decode
        ptr = (C.c_void_p, C.c_char_p)
        got = ["ptr" if t in ptr else t for t in fn.argtypes]
        assert got == ["ptr" if t in ptr else t for t in want_args], name
        assert fn.restype == want_ret, name


def test_product_code_never_reaches_the_oracle():
    """The package is the product: no module of bbscite_gb300/ imports the
    oracle (test infrastructure), and no native source includes or loads
    anything from oracle/.  Only tests, the smoke check and the bench's CPU
    baseline use it, as the checker."""
    import ast
    pkg = os.path.join(ROOT, "bbscite_gb300")
    for dirpath, _, files in os.walk(pkg):
        for fn in files:
            path = os.path.join(dirpath, fn)
            if fn.endswith(".py"):
                with open(path) as f:
                    tree = ast.parse(f.read(), path)
                for node in ast.walk(tree):
                    names = []
                    if isinstance(node, ast.Import):
                        names = [a.name for a in node.names]
                    elif isinstance(node, ast.ImportFrom):
                        names = [node.module or ""]
                    assert not any(n.split(".")[0] == "oracle"
                                   for n in names), path
            elif fn.endswith((".cu", ".cuh", ".h", ".cpp", ".hpp")):
                with open(path) as f:
                    text = f.read()
                assert not re.search(r'#include\s+[<"][^">]*oracle', text), path
                assert "libbbs_oracle" not in text and "liboracle" not in text, path


def _ring_distance(parent: np.ndarray) -> int:
    """The largest distance, in the canonical order (depth, then node
    index), from a node back to its parent: the ring of counts that rows of
    five to eight words inherit through must hold at least this many
    positions."""
    n = len(parent)
    root = n - 1
    depth = np.zeros(n, dtype=np.int64)
    for x in range(n):
        y, d = x, 0
        while y != root:
            y, d = int(parent[y]), d + 1
        depth[x] = d
    order = np.lexsort((np.arange(n), depth))
    pos = np.empty(n, dtype=np.int64)
    pos[order] = np.arange(n)
    return int(max(pos[x] - pos[parent[x]] for x in range(n) if x != root))


def test_random_trees_fit_the_ring():
    """Random trees of 131 to 256 nodes (uniform Pruefer codes, the chains'
    initial trees) fit the 64-entry ring: every node lies fewer than 64
    positions after its parent in the canonical order, so their counts are
    inherited without the masked-popcount fallback.  A star (every gene a
    child of the root) does not fit, and falls back."""
    rng = np.random.default_rng(2026)
    worst = 0
    for G in (130, 160, 200, 255):
        for _ in range(60):
            worst = max(worst, _ring_distance(D.random_parent_vector(rng, G)))
    assert worst < 64, worst
    star = np.full(256, 255, dtype=np.int64)
    assert _ring_distance(star) >= 64
