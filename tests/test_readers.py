"""File readers (tacogb_read_coo) against taco's own readers: each fixture file in
tests/golden was read by the taco CLI (readMTX / readTNS, then pack) and its CSR saved; the
records read here, packed by the oracle's restatement of taco's pack, must give the same CSR
bit for bit.  Host code only: no GPU."""
import os

import numpy as np
import pytest

import taco_gb300 as tg
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FILES = ["read_general.mtx", "read_symmetric.mtx", "read_array.mtx", "read_plain.tns"]


@pytest.mark.parametrize("name", FILES)
def test_reader_matches_taco(name):
    rows, cols, ri, ci, v = tg.read_coo(os.path.join(GOLDEN, name))
    g = np.load(os.path.join(GOLDEN, name.replace(".", "_") + ".npz"))
    pos, crd, vals = O.pack_csr(rows, cols, ri, ci, v)
    nr = len(g["pos"]) - 1
    assert np.array_equal(pos[:nr + 1], g["pos"]) and (pos[nr:] == pos[nr]).all()
    assert np.array_equal(crd, g["crd"]) and np.array_equal(vals, g["vals"])


def _write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_records_symmetric_order(tmp_path):
    """Off-diagonal entries are followed by their mirror, diagonal ones are not (taco's
    insertion order, src/storage/file_io_mtx.cpp:138-146); coordinates become 0-based."""
    f = _write(tmp_path, "s.mtx", "%%MatrixMarket matrix coordinate real symmetric\n% c\n"
                                  "3 3 3\n1 1 2.5\n3 1 -1\n\n3 2 4e-3\n")
    rows, cols, ri, ci, v = tg.read_coo(f)
    assert (rows, cols) == (3, 3)
    assert list(ri) == [0, 2, 0, 2, 1] and list(ci) == [0, 0, 2, 1, 2]
    assert list(v) == [2.5, -1.0, -1.0, 4e-3, 4e-3]


def test_records_array_and_tns(tmp_path):
    f = _write(tmp_path, "a.mtx", "%%MatrixMarket matrix array real general\n2 3\n"
                                  "1\n2\n3\n4\n5\n6\n")
    rows, cols, ri, ci, v = tg.read_coo(f)
    assert (rows, cols) == (2, 3)
    assert list(ri) == [0, 1, 0, 1, 0, 1] and list(ci) == [0, 0, 1, 1, 2, 2]  # column-major
    assert list(v) == [1, 2, 3, 4, 5, 6]
    f = _write(tmp_path, "t.tns", "2 3 1.5\n1 1 -2\n2 3 0.5\n")
    rows, cols, ri, ci, v = tg.read_coo(f)
    assert (rows, cols) == (2, 3) and list(ri) == [1, 0, 1] and list(v) == [1.5, -2.0, 0.5]


@pytest.mark.parametrize("text", [
    "%%MatrixMarket matrix coordinate pattern general\n2 2 1\n1 1\n",   # taco reads real only
    "%%MatrixMarket matrix coordinate real hermitian\n2 2 1\n1 1 1\n",
    "%%MatrixMarket matrix coordinate real general\n2 2 2\n1 1 1\n",     # fewer entries
    "%%MatrixMarket matrix coordinate real general\n2 2 1\n3 1 1\n",     # outside
    "%%MatrixMarket matrix coordinate real general\n2 2 1\n0 1 1\n",     # 0 in a 1-based file
    "%%MatrixMarket matrix coordinate real symmetric\n2 3 1\n1 1 1\n",   # not square
    "1 2 3 4.0\n",                                                       # 3-D .tns
])
def test_reader_rejects(tmp_path, text):
    with pytest.raises(tg.TacoGBError):
        tg.read_coo(_write(tmp_path, "bad.mtx" if text.startswith("%") else "bad.tns", text))


def test_reader_missing_file():
    with pytest.raises(tg.TacoGBError):
        tg.read_coo("/nonexistent/file.mtx")


@pytest.mark.parametrize("name", ["read_rua32.rb", "read_rhs.rb"])
def test_rutherford_boeing_csc(name):
    """tacogb_read_rb: taco's test matrix rua_32 (written again in this repository's own RB
    layout; the generator checked that taco's own rua_32.rb reads identically) and a matrix whose
    header announces right-hand sides (taco skips a fifth header line)."""
    g = np.load(os.path.join(GOLDEN, name.replace(".", "_") + ".npz"))
    rows, cols, colptr, rowidx, vals = tg.read_csc(os.path.join(GOLDEN, name))
    assert (rows, cols) == tuple(int(d) for d in g["dims"])
    assert np.array_equal(colptr, g["colptr"]) and np.array_equal(rowidx, g["rowidx"])
    assert np.array_equal(vals, g["cvals"])


def test_rutherford_boeing_matches_taco_csr():
    """The CSC of read_rua32.rb, transposed on the host, is the CSR taco's CLI made of
    rua_32.mtx."""
    g = np.load(os.path.join(GOLDEN, "read_rua32_rb.npz"))
    rows, cols, colptr, rowidx, vals = tg.read_csc(os.path.join(GOLDEN, "read_rua32.rb"))
    cr = np.repeat(np.arange(cols, dtype=np.int32), np.diff(colptr))
    o = np.lexsort((cr, rowidx))
    pos = np.searchsorted(rowidx[o], np.arange(rows + 1), side="left")
    assert np.array_equal(pos, g["pos"]) and np.array_equal(cr[o], g["crd"])
    assert np.array_equal(vals[o], g["vals"])


@pytest.mark.parametrize("text,what", [
    ("t k\n1 1 1 1 0\nRSA 3 3 1 0\n(1I1) (1I1) (1E1)\n1 1 2 2\n1\n1.0\n", "RUA"),
    ("t k\n4 1 1 2 0\nRUA 3 3 1 0\n(1I1) (1I1) (1E1)\n1 2 2 2\n1\n1.0\n", "shorter"),
    ("t k\n3 1 1 1 0\nRUA 3 3 2 0\n(1I1) (1I1) (1E1)\n1 2 2 3\n1 2\n1.0\n", "match"),
])
def test_rutherford_boeing_rejects(tmp_path, text, what):
    p = _write(tmp_path, "bad.rb", text)
    with pytest.raises(tg.TacoGBError) as e:
        tg.read_csc(p)
    assert what in str(e.value)
