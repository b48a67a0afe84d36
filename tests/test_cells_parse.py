"""The ASCII cell reader of the cone-octree build (mpf_cells_parse): the
reference reads an unsigned level and nine floats per cell."""
import numpy as np
import pytest

from conftest import load_golden


def test_parse_matches_float32_reads(pkg):
    g = load_golden("cells")
    text = str(g["cells_text"])
    rows = pkg.cells_parse(text)
    ref = np.array([l.split() for l in text.splitlines()], dtype=np.float32)
    assert rows.shape == (len(text.splitlines()), 10)
    np.testing.assert_array_equal(rows, ref)


def test_parse_rejects_malformed(pkg):
    with pytest.raises(pkg.MpfError):
        pkg.cells_parse("4 0.1 0.2\n")
    assert pkg.cells_parse("").shape == (0, 10)
