"""CPU tests of the C-ABI library: it loads, exports every declared symbol,
carries the reference's constant tables, and its host-side scheduling logic
is right.  No GPU compute is called here."""
import ctypes as C
import json
import os
import re

import numpy as np
import pytest

import mgldg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = json.load(open(os.path.join(ROOT, "tests", "golden", "master_tables.json")))


@pytest.fixture(scope="module", autouse=True)
def built():
    import importlib.util
    spec = importlib.util.spec_from_file_location("mgbuild", os.path.join(ROOT, "multigrid-ldg_gb300", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build(verbose=False)


def header_functions():
    src = open(os.path.join(ROOT, "include", "mgldg.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mgldg_\w+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    L = mgldg.lib()
    names = header_functions()
    assert len(names) >= 40
    for n in names:
        assert hasattr(L, n), n
    assert sorted(mgldg.EXPORTS) == names


@pytest.mark.parametrize("P", range(1, 7))
def test_library_tables_match_reference_constants(P):
    t = mgldg.master_tables(P)
    g = GOLDEN["tables"][str(P)]
    for key in ["nodes", "denom", "mass", "invmass", "diff"]:
        assert np.array_equal(np.asarray(t[key]).ravel(), np.array([float(s) for s in g[key]])), key
    q = GOLDEN["quadrature"]["10"]
    assert np.array_equal(t["quad_x"], np.array([float(s) for s in q["nodes"]]))
    assert np.array_equal(t["quad_w"], np.array([float(s) for s in q["weights"]]))


def morton_pattern(n):
    """5-point block pattern of an n x n grid in the reference's DFS (Morton) order."""
    def enc(ix, iy):
        e = 0
        for bit in range(16):
            e |= ((ix >> bit) & 1) << (2 * bit + 1)
            e |= ((iy >> bit) & 1) << (2 * bit)
        return e
    rows = [[] for _ in range(n * n)]
    for ix in range(n):
        for iy in range(n):
            e = enc(ix, iy)
            rows[e].append(e)
            for dx, dy in [(-1, 0), (1, 0), (0, -1), (0, 1)]:
                jx, jy = ix + dx, iy + dy
                if 0 <= jx < n and 0 <= jy < n:
                    rows[e].append(enc(jx, jy))
    rp = np.cumsum([0] + [len(r) for r in rows]).astype(np.int32)
    ci = np.concatenate([sorted(r) for r in rows]).astype(np.int32)
    return rp, ci


@pytest.mark.parametrize("n", [1, 2, 8, 32, 128])
def test_gs_wavefronts_on_morton_grid(n):
    # the forward sweep of an n x n grid in Morton order has 2n-1 levels
    rp, ci = morton_pattern(n)
    for rev in (False, True):
        lev, order, nl = mgldg.gs_levels(rp, ci, reverse=rev)
        assert nl == 2 * n - 1
        assert sorted(order.tolist()) == list(range(n * n))
        assert np.all(np.diff(lev[order]) >= 0)


def test_gs_levels_respect_sequential_order():
    # random symmetric pattern: every row's earlier neighbours sit on lower levels
    rng = np.random.default_rng(3)
    n = 200
    pairs = set()
    for _ in range(600):
        i, j = rng.integers(0, n, 2)
        if i != j:
            pairs.add((i, j)); pairs.add((j, i))
    rows = [[i] for i in range(n)]
    for i, j in pairs:
        rows[i].append(j)
    rp = np.cumsum([0] + [len(r) for r in rows]).astype(np.int32)
    ci = np.concatenate([sorted(r) for r in rows]).astype(np.int32)
    for rev in (False, True):
        lev, order, nl = mgldg.gs_levels(rp, ci, reverse=rev)
        for i in range(n):
            for j in rows[i]:
                if j == i:
                    continue
                earlier = j > i if rev else j < i
                if earlier:
                    assert lev[j] < lev[i]


@pytest.mark.parametrize("n", [2, 8, 32, 128])
@pytest.mark.parametrize("nsw", [1, 2, 3])
def test_gs_pass_depth_on_morton_grid(n, nsw):
    # nsw fused sweeps of an n x n Morton grid: sweep s trails sweep s-1 by
    # two levels, so the pass has 2n - 1 + 2 (nsw - 1) dependent steps
    rp, ci = morton_pattern(n)
    for rev in (False, True):
        lev, nl = mgldg.gs_pass_levels(rp, ci, nsw, reverse=rev)
        assert nl == 2 * n - 1 + 2 * (nsw - 1)
        lev1, _, nl1 = mgldg.gs_levels(rp, ci, reverse=rev)
        assert np.array_equal(lev[0], lev1) and nl1 == 2 * n - 1


def test_gs_pass_levels_respect_sweep_dependencies():
    # random symmetric pattern: sweep s of row i comes after sweep s of its
    # earlier neighbours and after sweep s-1 of itself and its later ones
    rng = np.random.default_rng(4)
    n, nsw = 150, 3
    pairs = set()
    for _ in range(400):
        i, j = rng.integers(0, n, 2)
        if i != j:
            pairs.add((i, j)); pairs.add((j, i))
    rows = [[i] for i in range(n)]
    for i, j in pairs:
        rows[i].append(j)
    rp = np.cumsum([0] + [len(r) for r in rows]).astype(np.int32)
    ci = np.concatenate([sorted(r) for r in rows]).astype(np.int32)
    for rev in (False, True):
        lev, nl = mgldg.gs_pass_levels(rp, ci, nsw, reverse=rev)
        assert nl == lev.max() + 1
        for s in range(nsw):
            for i in range(n):
                if s > 0:
                    assert lev[s - 1, i] < lev[s, i]
                for j in rows[i]:
                    if j == i:
                        continue
                    earlier = j > i if rev else j < i
                    if earlier:
                        assert lev[s, j] < lev[s, i]
                    elif s > 0:
                        assert lev[s - 1, j] < lev[s, i]


def test_context_creation_without_gpu_fails_cleanly():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    h = C.c_void_p()
    rc = mgldg.lib().mgldg_ctx_create(0, C.byref(h))
    assert rc == mgldg.ERR_CUDA and not h.value
