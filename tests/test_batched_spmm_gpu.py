"""Batched SpMM parity on the GPU: C_m = A_m B_m for many uneven CSR matrices in one persistent
graph-captured launch, every C_m against the oracle (taco's serial loop restated in C).

Bars (normwise relative error per matrix, against the FP64 oracle): FP64 native and
double-float 1e-12; FP32 native 1e-5, compensated FP32 1e-6; FP32 values with BF16 B 1e-5
against the oracle evaluated on the BF16-rounded B (FP32 accumulation; the rounding of B itself,
about 4e-3, is the single-matrix tests' concern).  Re-running a plan is bitwise identical.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import taco_gb300 as tg  # noqa: E402
from oracle import oracle as O  # noqa: E402
from taco_gb300 import workloads as W  # noqa: E402
from tests.helpers import normwise  # noqa: E402

pytestmark = pytest.mark.gpu
TOL = {("f64", 0): 1e-12, ("f64", 1): 1e-12, ("f32", 0): 1e-6, ("f32", 1): 1e-5,
       ("bf16", 0): 1e-5}


def _mats():
    rng = np.random.default_rng(21)
    out = [(np.zeros(1, np.int32), np.zeros(0, np.int32), np.zeros(0), 6),
           (np.zeros(40, np.int32), np.zeros(0, np.int32), np.zeros(0), 8)]
    cols = 9000  # one row over many tiles between short rows
    lens = rng.integers(0, 4, 700).astype(np.int32)
    lens[350] = cols
    pos = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    crd = np.concatenate([np.arange(cols) if n == cols else np.sort(rng.choice(cols, n, False))
                          for n in lens])
    out.append((pos, crd.astype(np.int32), rng.uniform(-1, 1, len(crd)), cols))
    for m in range(18):
        s = W.batch_spec(m, seed=77, rows_hi=6000)
        p, c, v = W.generate(s)
        out.append((p, c, v, s.cols))
    return out


MATS = _mats()


def _run(kind, precision, N, reps=2):
    vt = torch.float64 if kind == "f64" else torch.float32
    bt = {"f64": torch.float64, "f32": torch.float32, "bf16": torch.bfloat16}[kind]
    mats, Bs, Cs, refs = [], [], [], []
    for m, (pos, crd, vals, cols) in enumerate(MATS):
        mats.append(tg.CsrMatrix.from_numpy(pos, crd, vals, cols, dtype=vt))
        B = W.dense(900 + m, cols * N).reshape(cols, N)
        Bd = torch.from_numpy(B).to("cuda", bt)
        Bs.append(Bd)
        Cs.append(torch.full((len(pos) - 1, N), float("nan"), dtype=vt, device="cuda"))
        refs.append(O.spmm(pos, crd, vals, Bd.double().cpu().numpy() if kind == "bf16" else B))
    plan = tg.SpmmBatch(mats, Bs, Cs, precision=precision)
    outs = []
    for _ in range(reps):
        plan.run()
        torch.cuda.synchronize()
        outs.append([c.double().cpu().numpy() for c in Cs])
    for a, b in zip(outs[0], outs[-1]):
        assert np.array_equal(a, b, equal_nan=True)
    cyc = plan.matrix_cycles()
    plan.close()
    return outs[0], refs, cyc


@pytest.mark.parametrize("kind,precision", sorted(TOL))
@pytest.mark.parametrize("N", [32, 48, 64])
def test_batched_spmm(kind, precision, N):
    Cs, refs, cyc = _run(kind, precision, N)
    tol = TOL[(kind, precision)]
    for m, (C, ref) in enumerate(zip(Cs, refs)):
        assert C.shape == ref.shape
        assert normwise(C, ref) <= tol, m
    assert cyc.shape == (len(MATS),) and np.all(cyc[3:] > 0)


def test_batched_spmm_f32_against_rounded_inputs():
    """Compensated FP32 against the FP64 oracle on the FP32-rounded inputs: 1e-7."""
    Cs, _, _ = _run("f32", 0, 32)
    for m, (pos, crd, vals, cols) in enumerate(MATS):
        B = W.dense(900 + m, cols * 32).reshape(cols, 32)
        ref = O.spmm(pos, crd, vals.astype(np.float32).astype(np.float64),
                     B.astype(np.float32).astype(np.float64))
        assert normwise(Cs[m], ref) <= 1e-7, m


def test_batched_spmm_rejects_mixed_types():
    A = tg.CsrMatrix.from_numpy(*MATS[3][:3], MATS[3][3])
    B = torch.zeros(MATS[3][3], 32, dtype=torch.float32, device="cuda")
    C = torch.zeros(len(MATS[3][0]) - 1, 32, dtype=torch.float64, device="cuda")
    with pytest.raises(tg.TacoGBError):
        tg.SpmmBatch([A], [B], [C])
