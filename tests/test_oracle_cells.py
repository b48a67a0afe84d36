"""CPU tests: the C oracle's cone octree build from ASCII cells
(oracle/mpf_oracle_cells.c: Input::importascii + Miscellaneous::correctOctree)
against the reference's own build of the same files
(tests/golden/cells.npz, tests/golden/cells_sparse.npz):

* every correction option (correction, coarsecorrection, acorrection with
  its amin) and the three interpolation orders of the completed children:
  the same cells, keys and 48-byte records;
* many incomplete octs whose appended children read one another: the
  reference's sequential appends and the device's order (waves of gathers
  that read only children of earlier waves, then the rest in order) give the
  same records, and the waves take the counts the device reports.

The last record in key order is left out of the field comparison: the
reference's SimpleHyperOctree::update (simplehyperoctree.h:1286-1303) reads
one element past its container for it."""
import importlib

import numpy as np
import pytest

from conftest import load_golden

CORRECTIONS = {"full": (1, 1, 0, 2), "nocorr": (0, 0, 0, 2), "nocorr_coarse": (0, 1, 0, 2), "corr_nocoarse": (1, 0, 0, 2),
               "acorr": (1, 1, 1, 2), "nocorr_acorr": (0, 0, 1, 2), "full_o1": (1, 1, 0, 1), "full_o0": (1, 1, 0, 0)}
FIELDS = ("dphidt", "a", "dphidx", "dphidy", "dphidz", "phi", "rho")


def _records(b):
    S = importlib.import_module("magrathea-pathfinder_gb300.synth")
    return np.frombuffer(b.tobytes(), dtype=S.RECORD)


def _build(oracle_mod, g, rows, **kw):
    cos = {"t": g["cosmo_t"], "a": g["cosmo_a"], "dadt": g["cosmo_dadt"]}
    return oracle_mod.cells_build(rows, cos, g["cone7"], g["sphere4"], float(g["h"]), float(g["lboxmpch"]),
                                  float(g["mpc"]), **kw)


def _assert_same(rec, ref_bytes):
    got, ref = _records(rec), _records(ref_bytes)
    assert got.shape == ref.shape, (got.shape, ref.shape)
    np.testing.assert_array_equal(got["hi"], ref["hi"])
    np.testing.assert_array_equal(got["lo"], ref["lo"])
    for name in FIELDS:
        np.testing.assert_array_equal(got[name][:-1].view(np.uint32), ref[name][:-1].view(np.uint32), err_msg=name)


@pytest.fixture(scope="module")
def cells():
    return load_golden("cells")


@pytest.fixture(scope="module")
def sparse():
    return load_golden("cells_sparse")


def test_parse_reads_the_rows(oracle_mod, cells):
    rows = oracle_mod.cells_parse(str(cells["cells_text"]))
    assert rows.shape[1] == 10 and rows.shape[0] > 1000
    lines = str(cells["cells_text"]).split("\n")
    first = lines[0].split()
    assert rows[0, 0] == int(first[0]) and rows[0, 9] == np.float32(first[9])
    with pytest.raises(ValueError):
        oracle_mod.cells_parse("7 0.1 0.2 x")


@pytest.mark.parametrize("name", sorted(CORRECTIONS))
def test_build_equals_reference(oracle_mod, cells, name):
    corr, coarse, acorr, order = CORRECTIONS[name]
    rows = oracle_mod.cells_parse(str(cells["cells_text"]))
    rec, amin, info = _build(oracle_mod, cells, rows, order=order, correction=bool(corr), coarsecorrection=bool(coarse),
                             acorrection=bool(acorr))
    _assert_same(rec, cells["ref_records_" + name])
    if acorr:
        assert amin == float(cells["ref_amin_" + name])
    if corr:
        assert info["incomplete"] > 0 and info["sequential"] == 8 * info["incomplete"]


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("waves", [0, 1, 2, 32])
def test_completion_order_does_not_change_the_records(oracle_mod, sparse, order, waves):
    rows = oracle_mod.cells_parse(str(sparse["cells_text"]))
    rec, _, info = _build(oracle_mod, sparse, rows, order=order, completion_waves=waves)
    _assert_same(rec, sparse["ref_records_o%d" % order])
    assert info["incomplete"] == 615
    assert info["in_waves"] + info["sequential"] == 8 * 615
    if waves == 0:
        assert info["in_waves"] == 0
    elif waves == 1:
        # some children read children appended before them: they wait for a second wave
        assert info["waves"] == 1 and info["sequential"] > 0
    else:
        assert info["waves"] == 2 and info["sequential"] == 0


def test_rotation_and_coarse_only(oracle_mod, cells):
    """A narrow cone's rotation applied to the rows equals the rows rotated
    beforehand; coarseonly keeps the coarse file level alone."""
    rows = oracle_mod.cells_parse(str(cells["cells_text"]))
    th = 0.3
    rot = np.array([[np.cos(th), -np.sin(th), 0.0], [np.sin(th), np.cos(th), 0.0], [0.0, 0.0, 1.0]])
    turned = rows.copy()
    for cols in ((1, 2, 3), (6, 7, 8)):
        v = rows[:, cols].astype(np.float64)
        turned[:, cols] = (v[:, 0:1] * rot[:, 0] + v[:, 1:2] * rot[:, 1] + v[:, 2:3] * rot[:, 2]).astype(np.float32)
    a, _, _ = _build(oracle_mod, cells, rows, rotm1=rot)
    b, _, _ = _build(oracle_mod, cells, turned)
    np.testing.assert_array_equal(a, b)
    coarse = int(rows[:, 0].min())
    c, _, _ = _build(oracle_mod, cells, rows, coarseonly=True, ncoarse=coarse, coarsecorrection=False)
    assert 0 < c.shape[0] // 48 < a.shape[0] // 48


def test_rotated_build_equals_reference(oracle_mod, sparse):
    """A narrow cone's rotation of the cells' positions and forces
    (importascii's rotm1, input.h:1034-1039) against the reference's rotated
    build of the same file."""
    rows = oracle_mod.cells_parse(str(sparse["cells_text"]))
    rec, _, _ = _build(oracle_mod, sparse, rows, rotm1=sparse["rotm1"], completion_waves=32)
    _assert_same(rec, sparse["ref_records_rot"])
