"""The fixtures of taco's own API into the library (tests/golden/taco_dropin_<p>.npz, replayed on
a GPU by tests/test_taco_dropin_gpu.py) checked on the CPU: taco's result in each equals the
oracle's restatement on the recorded operands, and the packs have taco's layouts.  With
TACO_REFERENCE naming taco's source tree, the fixtures are also made again from genuine taco
(taco::Tensor statements, compileSource with the forwarding source, assemble, compute) and must
describe the same statements."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import normwise

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _load(p):
    return np.load(os.path.join(GOLDEN, "taco_dropin_%s.npz" % p))


def _hdr(g, k):
    h = [int(v) for v in g["a%d_hdr" % k]]
    order = h[0]
    return {"order": order, "csize": h[1], "dims": h[2:2 + order],
            "ordering": h[2 + order:2 + 2 * order], "types": h[2 + 2 * order:]}


@pytest.mark.parametrize("p", ["spmv", "spmm", "spgemm"])
def test_fixture_layouts(p):
    g = _load(p)
    A = _hdr(g, 1)
    assert A["types"] == [0, 1] and A["ordering"] == [0, 1] and A["csize"] == 64  # CSR, FP64
    B, R = _hdr(g, 2), _hdr(g, 0)
    assert B["types"] == ([0, 1] if p == "spgemm" else [0] * B["order"])
    assert R["types"] == ([0, 1] if p == "spgemm" else [0] * R["order"])
    assert g["a1_pos1"][0] == 0 and g["a1_pos1"][-1] == len(g["a1_crd1"])


@pytest.mark.parametrize("p", ["spmv", "spmm", "spgemm"])
def test_fixture_results_match_oracle(p):
    g = _load(p)
    pos, crd, vals = g["a1_pos1"], g["a1_crd1"], g["a1_vals"]
    if p == "spmv":
        assert normwise(O.spmv(pos, crd, vals, g["a2_vals"]), g["e_vals"]) <= 1e-12
    elif p == "spmm":
        dims = _hdr(g, 2)["dims"]
        Bm = g["a2_vals"].reshape(dims)
        assert normwise(O.spmm(pos, crd, vals, Bm).ravel(), g["e_vals"]) <= 1e-12
    else:
        ref = O.spgemm(pos, crd, vals, g["a2_pos1"], g["a2_crd1"], g["a2_vals"],
                       _hdr(g, 2)["dims"][1])
        assert np.array_equal(ref[0], g["e_pos1"]) and np.array_equal(ref[1], g["e_crd1"])
        assert np.array_equal(ref[2], g["e_vals"])


@pytest.mark.skipif(not os.environ.get("TACO_REFERENCE"),
                    reason="TACO_REFERENCE does not name taco's source tree")
def test_fixtures_regenerate_from_genuine_taco(tmp_path, monkeypatch):
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    monkeypatch.setattr(mg, "OUT", str(tmp_path))
    mg.dropin_cases(os.environ["TACO_REFERENCE"])
    for p in ("spmv", "spmm", "spgemm"):
        new = np.load(os.path.join(str(tmp_path), "taco_dropin_%s.npz" % p))
        old = _load(p)
        assert sorted(new.files) == sorted(old.files)
        for k in old.files:
            assert new[k].shape == old[k].shape, (p, k)
