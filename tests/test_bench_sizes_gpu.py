"""Parity at the sizes the benchmark measures: every configuration bench.py times is checked here
on the same generator specs, against the oracle (taco's loops restated in C).

  SpMV  65,536^2, row lengths uniform on [4,28]: every variant, FP64 and compensated FP32, all
        rows against the oracle.
  SpMM  1,048,576^2 power-law (mean 32, max 10,000), N = 64 and 256, FP64, FP32 and BF16 B:
        the whole product is computed on the GPU; the oracle recomputes a sample of rows (the
        64 longest, which span many merge tiles, the first and last, and 20,000 random rows).
  Batched SpMV and SpMM  matrices of the 4,096-matrix benchmark batch (same specs, same seed):
        its largest matrices (by nonzeros and by rows) and a random selection, FP64 plans and compensated
        FP32 plans with the learned kinds, every matrix against the FP64 oracle.

Bars (normwise relative error against the FP64 oracle): FP64 1e-12; compensated FP32 1e-6 (and
1e-7 against the oracle on the FP32-rounded inputs for SpMV); SpMM BF16 B with FP32 accumulation
1e-2 against the FP64 oracle and 1e-5 against the oracle on the rounded inputs.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import taco_gb300 as tg  # noqa: E402
from oracle import oracle as O  # noqa: E402
from taco_gb300 import workloads as W  # noqa: E402
from tests.helpers import normwise, sample_rows, sub_rows  # noqa: E402

pytestmark = pytest.mark.gpu
F64_TOL = 1e-12
F32C_TOL = 1e-6
F32C_ROUNDED_TOL = 1e-7
BF16_TOL = 1e-2
BF16_ROUNDED_TOL = 1e-5


def _spmv_variants():
    return [-1] + list(range(tg.lib().tacogb_spmv_variant_count()))


# ------------------------------------------------------------------------ SpMV 65,536^2

@pytest.fixture(scope="module")
def spmv_small():
    s = W.spmv_small()
    pos, crd, vals = W.generate(s)
    x = W.dense(23, s.cols)  # bench.py's x
    return s, pos, crd, vals, x, O.spmv(pos, crd, vals, x)


def test_spmv_small_f64_every_variant(spmv_small):
    s, pos, crd, vals, x, ref = spmv_small
    A = tg.CsrMatrix.from_numpy(pos, crd, vals, s.cols)
    xd = torch.from_numpy(x).cuda()
    for v in _spmv_variants():
        y = tg.spmv(A, xd, variant=v).cpu().numpy()
        assert normwise(y, ref) <= F64_TOL, v


def test_spmv_small_f32_compensated(spmv_small):
    s, pos, crd, vals, x, ref = spmv_small
    A = tg.CsrMatrix.from_numpy(pos, crd, vals, s.cols, dtype=torch.float32)
    xd = torch.from_numpy(x).to("cuda", torch.float32)
    ref32 = O.spmv(pos, crd, vals.astype(np.float32).astype(np.float64),
                   x.astype(np.float32).astype(np.float64))
    for v in _spmv_variants():
        y = tg.spmv(A, xd, variant=v).double().cpu().numpy()
        assert normwise(y, ref) <= F32C_TOL, v
        assert normwise(y, ref32) <= F32C_ROUNDED_TOL, v


# ------------------------------------------------------------------------ SpMM 1,048,576^2

@pytest.fixture(scope="module")
def spmm_matrix():
    s = W.spmm_powerlaw()
    pos, crd, vals = W.generate(s)
    idx = sample_rows(pos, 20000, seed=3)
    return s, pos, crd, vals, idx, sub_rows(pos, crd, vals, idx)


@pytest.mark.parametrize("N", [64, 256])
@pytest.mark.parametrize("kind", ["f64", "f32", "bf16"])
def test_spmm_powerlaw_full_size(spmm_matrix, N, kind):
    s, pos, crd, vals, idx, (spos, scrd, svals) = spmm_matrix
    B = W.dense(29, s.cols * N).reshape(s.cols, N)  # bench.py's B
    vt = torch.float64 if kind == "f64" else torch.float32
    bt = {"f64": torch.float64, "f32": torch.float32, "bf16": torch.bfloat16}[kind]
    A = tg.CsrMatrix.from_numpy(pos, crd, vals, s.cols, dtype=vt)
    Bd = torch.from_numpy(B).to("cuda", bt)
    C = tg.spmm(A, Bd)
    Cs = C[torch.from_numpy(idx).cuda()].double().cpu().numpy()
    assert not np.isnan(Cs).any()
    ref = O.spmm(spos, scrd, svals, B)
    err = normwise(Cs, ref)
    if kind == "f64":
        assert err <= F64_TOL
    elif kind == "f32":
        assert err <= F32C_TOL
    else:
        assert err <= BF16_TOL
        Br = Bd.double().cpu().numpy()
        ref_r = O.spmm(spos, scrd, svals.astype(np.float32).astype(np.float64), Br)
        assert normwise(Cs, ref_r) <= BF16_ROUNDED_TOL
    del C, Bd, A
    torch.cuda.empty_cache()


# ------------------------------------------------------------------------ batched

def _bench_batch_subset(count_random=120, largest=6, seed=5):
    """Indices into the benchmark batch: its `largest` matrices by expected nonzeros and
    `count_random` others."""
    specs = [W.batch_spec(m) for m in range(4096)]
    size = np.array([s.rows * s.mean for s in specs])
    rows = np.array([s.rows for s in specs])
    big = np.union1d(np.argsort(size, kind="stable")[-largest:],
                     np.argsort(rows, kind="stable")[-2:])
    rest = np.setdiff1d(np.arange(4096), big)
    rnd = np.random.default_rng(seed).choice(rest, count_random, replace=False)
    idx = np.sort(np.concatenate([big, rnd]))
    return idx, [specs[m] for m in idx]


@pytest.fixture(scope="module")
def bench_batch():
    idx, specs = _bench_batch_subset()
    mats = []
    for m, s in zip(idx, specs):
        pos, crd, vals = W.generate(s)
        mats.append((int(m), s, pos, crd, vals))
    assert max(s.rows for _, s, *_ in mats) == max(W.batch_spec(m).rows for m in range(4096))
    return mats


def test_batched_spmv_bench_matrices(bench_batch):
    from taco_gb300 import autotune as AT
    dev64, dev32, xs64, xs32, ys64, ys32, refs, refs32 = [], [], [], [], [], [], [], []
    for m, s, pos, crd, vals in bench_batch:
        x = W.dense(1000 + m, s.cols)
        dev64.append(tg.CsrMatrix.from_numpy(pos, crd, vals, s.cols))
        dev32.append(tg.CsrMatrix.from_numpy(pos, crd, vals, s.cols, dtype=torch.float32))
        xs64.append(torch.from_numpy(x).cuda())
        xs32.append(xs64[-1].float())
        ys64.append(torch.full((s.rows,), float("nan"), dtype=torch.float64, device="cuda"))
        ys32.append(torch.full((s.rows,), float("nan"), dtype=torch.float32, device="cuda"))
        refs.append(O.spmv(pos, crd, vals, x))
        refs32.append(O.spmv(pos, crd, vals.astype(np.float32).astype(np.float64),
                             x.astype(np.float32).astype(np.float64)))
    plan64 = tg.SpmvBatch(dev64, xs64, ys64, precision=0)
    kinds = AT.learned_select(AT.load_model(), dev32)
    plan32 = tg.SpmvBatch(dev32, xs32, ys32, precision=0, variants=kinds)
    for plan in (plan64, plan32):
        plan.run()
    torch.cuda.synchronize()
    for k in range(len(bench_batch)):
        y64, y32 = ys64[k].cpu().numpy(), ys32[k].double().cpu().numpy()
        assert normwise(y64, refs[k]) <= F64_TOL, k
        assert normwise(y32, refs[k]) <= F32C_TOL, k
        assert normwise(y32, refs32[k]) <= F32C_ROUNDED_TOL, k
    plan64.close()
    plan32.close()


def test_batched_spmm_bench_matrices(bench_batch):
    N = 32
    mats = bench_batch[::4]  # the batched SpMM keeps a dense B and C per matrix: a quarter
    for low in (False, True):
        vt = torch.float32 if low else torch.float64
        dev, Bs, Cs, refs, sel = [], [], [], [], []
        for m, s, pos, crd, vals in mats:
            B = W.dense(2000 + m, s.cols * N).reshape(s.cols, N)
            dev.append(tg.CsrMatrix.from_numpy(pos, crd, vals, s.cols, dtype=vt))
            Bs.append(torch.from_numpy(B).to("cuda", vt))
            Cs.append(torch.full((s.rows, N), float("nan"), dtype=vt, device="cuda"))
            k = sample_rows(pos, 2000, seed=m, longest=16)
            sel.append(k)
            refs.append(O.spmm(*sub_rows(pos, crd, vals, k), B))
        plan = tg.SpmmBatch(dev, Bs, Cs, precision=0)
        plan.run()
        torch.cuda.synchronize()
        for j in range(len(mats)):
            Cj = Cs[j][torch.from_numpy(sel[j]).cuda()].double().cpu().numpy()
            assert normwise(Cj, refs[j]) <= (F32C_TOL if low else F64_TOL), j
        plan.close()
