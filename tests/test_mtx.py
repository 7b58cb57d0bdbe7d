"""MatrixMarket input and the demo harness."""
import io

import numpy as np
import pytest

from sympiler_gb300 import matgen as mg
from sympiler_gb300.mtx import MtxError, lower_triangle, read_mtx, write_mtx


def _write(tmp_path, text, name="m.mtx"):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_symmetric_lower_stored_and_upper_stored_agree(tmp_path):
    A = mg.lap2d(12)
    L = mg.tril(A)
    lo = str(tmp_path / "lo.mtx")
    write_mtx(lo, L, symmetric=True, comment="lower triangle stored")
    U = mg.transpose(L)  # same symmetric matrix, upper triangle stored
    up = str(tmp_path / "up.mtx")
    write_mtx(up, U, symmetric=True)
    for path in (lo, up):
        Lr, Lc = lower_triangle(path)
        assert np.array_equal(Lr.p, L.p) and np.array_equal(Lr.i, L.i) and np.array_equal(Lr.x, L.x)
        T = mg.transpose(L)
        assert np.array_equal(Lc.p, T.p) and np.array_equal(Lc.i, T.i) and np.array_equal(Lc.x, T.x)


def test_general_file_keeps_entries_on_and_below_the_diagonal(tmp_path):
    A = mg.convdiff3d(4)  # nonsymmetric
    path = str(tmp_path / "g.mtx")
    write_mtx(path, A)
    Lr, _ = lower_triangle(path)
    want = mg.tril(A)
    assert np.array_equal(Lr.p, want.p) and np.array_equal(Lr.i, want.i) and np.array_equal(Lr.x, want.x)


def test_pattern_comments_and_entry_order(tmp_path):
    text = ("%%MatrixMarket matrix coordinate pattern symmetric\n"
            "% a comment\n%\n"
            "3 3 5\n"
            "3 3\n2 1\n1 1\n3 2\n2 2\n")
    nr, nc, r, c, v, sym = read_mtx(_write(tmp_path, text))
    assert (nr, nc, sym) == (3, 3, "symmetric") and np.all(v == 1.0)
    L, _ = lower_triangle(_write(tmp_path, text, "p.mtx"))
    assert list(L.p) == [0, 1, 3, 5] and list(L.i) == [0, 0, 1, 1, 2]


@pytest.mark.parametrize("text,msg", [
    ("%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n", "coordinate"),
    ("%%MatrixMarket matrix coordinate complex general\n1 1 1\n1 1 1 0\n", "complex"),
    ("%%MatrixMarket matrix coordinate real general\n2 3 1\n1 1 1\n", "square"),
    ("%%MatrixMarket matrix coordinate real general\n2 2 1\n1 1 1\n", "diagonal"),
    ("%%MatrixMarket matrix coordinate real general\n2 2 2\n1 1 1\n", "declared"),
    ("not a header\n", "header"),
])
def test_bad_files_are_rejected(tmp_path, text, msg):
    with pytest.raises(MtxError, match=msg):
        lower_triangle(_write(tmp_path, text))


@pytest.mark.gpu
def test_demo_harness_on_a_file_and_random_mode(gpu, tmp_path):
    from sympiler_gb300 import sptrsv_demo
    A = mg.lap2d(100)
    path = str(tmp_path / "lap2d_100.mtx")
    write_mtx(path, mg.tril(A), symmetric=True)
    buf = io.StringIO()
    assert sptrsv_demo.run(path, -1, 4000, parts=8, header=True, out=buf) == 0
    head, row = buf.getvalue().strip().split("\n")
    assert head == sptrsv_demo.HEADER
    f = row.split(",")
    assert f[0] == "lap2d_100.mtx" and f[1] == "No" and f[2] == "8"
    assert all(float(t) > 0 for t in f[5:9])
    buf = io.StringIO()
    assert sptrsv_demo.run(None, out=buf) == 0
    assert buf.getvalue().startswith("Random_16,No,")
