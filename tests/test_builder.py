"""Block-by-block assembly with the reference's SparseBlockMatrix calls
(mgldg_bsr_builder_*: reset, setBlock, addToBlock, blockExists, nnzb;
sparseblockmatrix.tpp:79-127) against a plain dictionary model that applies
the same calls: setBlock overwrites, addToBlock sums in call order, so every
exported block equals the model's bit for bit.  The upload (finalize) is a
GPU test.
"""
import numpy as np
import pytest

mgldg = pytest.importorskip("mgldg")


def _lib_or_skip():
    try:
        mgldg.lib()
    except RuntimeError as e:
        pytest.skip(str(e))


def _random_assembly(seed, nbr=7, nbc=5, br=3, bc=2, ncalls=300):
    rng = np.random.default_rng(seed)
    b = mgldg.BlockBuilder(nbr, nbc, br, bc)
    model = {}
    for _ in range(ncalls):
        i, j = int(rng.integers(nbr)), int(rng.integers(nbc))
        blk = rng.standard_normal((br, bc))
        if rng.random() < 0.25:
            b.set_block(i, j, blk)
            model[(i, j)] = blk.copy()
        else:
            b.add_to_block(i, j, blk)
            model[(i, j)] = model[(i, j)] + blk if (i, j) in model else blk.copy()
    return b, model


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_builder_matches_the_reference_semantics(seed):
    _lib_or_skip()
    b, model = _random_assembly(seed)
    assert b.nnzb() == len(model)
    rp, ci, v = b.export()
    keys = sorted(model)
    assert np.array_equal(rp, np.searchsorted([k[0] for k in keys], np.arange(len(rp)), side="left"))
    assert [(int(np.searchsorted(rp, q, side="right") - 1), int(c)) for q, c in enumerate(ci)] == keys
    for q, k in enumerate(keys):
        assert np.array_equal(v[q], model[k])          # bit for bit: same additions in the same order
    for i in range(7):
        for j in range(5):
            assert b.block_exists(i, j) == ((i, j) in model)


def test_builder_rejects_bad_calls():
    _lib_or_skip()
    b = mgldg.BlockBuilder(2, 3, 2, 2)
    for i, j in ((-1, 0), (2, 0), (0, 3), (0, -1)):
        with pytest.raises(mgldg.MgldgError):
            b.add_to_block(i, j, np.ones(4))
        with pytest.raises(mgldg.MgldgError):
            b.block_exists(i, j)
    with pytest.raises(ValueError):
        b.set_block(0, 0, np.ones(3))
    with pytest.raises(mgldg.MgldgError):
        mgldg.BlockBuilder(2, 2, 0, 2)
    empty = mgldg.BlockBuilder(3, 3, 2, 2)
    rp, ci, v = empty.export()
    assert empty.nnzb() == 0 and np.array_equal(rp, np.zeros(4)) and len(ci) == 0


@pytest.mark.gpu
def test_builder_finalize_uploads_the_exported_matrix(ctx):
    b, model = _random_assembly(4)
    rp, ci, v = b.export()
    A = b.finalize(ctx)
    rp2, ci2, v2 = A.download()
    assert np.array_equal(rp, rp2) and np.array_equal(ci, ci2) and np.array_equal(v, v2)
