"""Batched SpMV parity on the GPU: one persistent graph-captured launch over many uneven CSR
matrices, every matrix's y against the oracle (taco's serial loop restated in C).

Bars: FP64 (double-float or native accumulation) within 1e-12 normwise relative error per
matrix; FP32 values with compensated accumulation within 1e-6 of the FP64 oracle and within
1e-7 of the FP64 oracle on the FP32-rounded inputs.  Re-running a plan is bitwise identical
(the work queue resets itself; carries are summed in tile order).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import taco_gb300 as tg  # noqa: E402
from oracle import oracle as O  # noqa: E402
from taco_gb300 import workloads as W  # noqa: E402
from tests.helpers import normwise  # noqa: E402

pytestmark = pytest.mark.gpu
F64_TOL = 1e-12
F32_TOL = 1e-6
F32_COMP_TOL = 1e-7
KINDS = tg.batch_variants() if torch.cuda.is_available() else []


def _edge_set():
    rng = np.random.default_rng(11)
    out = []
    out.append((np.zeros(1, np.int32), np.zeros(0, np.int32), np.zeros(0), 7))  # 0 rows
    out.append((np.zeros(301, np.int32), np.zeros(0, np.int32), np.zeros(0), 9))  # no nonzeros
    out.append((np.array([0, 3], np.int32), np.array([0, 4, 9], np.int32),
                np.array([1.0, -2.0, 0.5]), 10))  # one row
    cols = 20000  # one row over many merge tiles between short rows
    lens = np.ones(1000, np.int32)
    lens[500] = cols
    pos = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    crd = np.concatenate([np.arange(cols) if n == cols else rng.choice(cols, 1) for n in lens])
    out.append((pos, crd.astype(np.int32), rng.uniform(-1, 1, len(crd)), cols))
    lens = rng.integers(0, 3, 5000).astype(np.int32)  # mostly empty or single
    pos = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    crd = np.concatenate([np.sort(rng.choice(4000, n, replace=False)) for n in lens])
    out.append((pos, crd.astype(np.int32), rng.uniform(-1, 1, len(crd)), 4000))
    return out


def _generated_set(count, rows_hi=20000):
    out = []
    for m in range(count):
        s = W.batch_spec(m, rows_hi=rows_hi)
        pos, crd, vals = W.generate(s)
        out.append((pos, crd, vals, s.cols))
    return out


def _run(mats_np, dtype, precision=0, variants=None, reps=2):
    mats, xs, ys, xs_np = [], [], [], []
    for m, (pos, crd, vals, cols) in enumerate(mats_np):
        mats.append(tg.CsrMatrix.from_numpy(pos, crd, vals, cols, dtype=dtype))
        x = W.dense(100 + m, cols)
        xs_np.append(x)
        xs.append(torch.from_numpy(x).to("cuda", dtype))
        ys.append(torch.full((len(pos) - 1,), float("nan"), dtype=dtype, device="cuda"))
    plan = tg.SpmvBatch(mats, xs, ys, precision=precision, variants=variants)
    outs = []
    for _ in range(reps):
        plan.run()
        torch.cuda.synchronize()
        outs.append([y.double().cpu().numpy() for y in ys])
    plan.close()
    for a, b in zip(outs[0], outs[-1]):
        assert np.array_equal(a, b, equal_nan=True)
    return outs[0], xs_np


def _check(mats_np, ys, xs_np, tol, f32=False):
    for m, (pos, crd, vals, cols) in enumerate(mats_np):
        ref = O.spmv(pos, crd, vals, xs_np[m])
        assert ys[m].shape == ref.shape
        assert normwise(ys[m], ref) <= tol, m
        if f32:
            v32 = vals.astype(np.float32).astype(np.float64)
            x32 = xs_np[m].astype(np.float32).astype(np.float64)
            assert normwise(ys[m], O.spmv(pos, crd, v32, x32)) <= F32_COMP_TOL, m


@pytest.mark.parametrize("kind", range(len(KINDS)))
@pytest.mark.parametrize("precision", [0, 1])
def test_edge_batch_f64(kind, precision):
    mats = _edge_set()
    ys, xs = _run(mats, torch.float64, precision, [kind] * len(mats))
    _check(mats, ys, xs, F64_TOL)


@pytest.mark.parametrize("kind", range(len(KINDS)))
def test_edge_batch_f32(kind):
    mats = _edge_set()
    ys, xs = _run(mats, torch.float32, 0, [kind] * len(mats))
    _check(mats, ys, xs, F32_TOL, f32=True)


@pytest.fixture(scope="module")
def generated():
    return _generated_set(60)


@pytest.mark.parametrize("precision", [0, 1])
def test_generated_batch_mixed_kinds_f64(generated, precision):
    variants = [m % len(KINDS) for m in range(len(generated))]
    ys, xs = _run(generated, torch.float64, precision, variants)
    _check(generated, ys, xs, F64_TOL)


def test_generated_batch_default_kind_f32(generated):
    ys, xs = _run(generated, torch.float32)
    _check(generated, ys, xs, F32_TOL, f32=True)


def test_unaligned_arrays_fall_back_to_vector_units(generated):
    """Arrays that are not 16-byte aligned cannot be staged with bulk copies; merge kinds are
    planned as vector units for them and the results stay exact."""
    mats, xs, ys, refs = [], [], [], []
    for m, (pos, crd, vals, cols) in enumerate(generated[:6]):
        p = torch.from_numpy(np.concatenate([pos[:1], pos])).cuda()[1:]  # offset by 4 bytes
        c = torch.from_numpy(np.concatenate([pos[:1], crd])).cuda()[1:]
        v = torch.from_numpy(np.concatenate([vals[:1], vals])).cuda()[1:]
        mats.append(tg.CsrMatrix(p, c, v, cols))
        x = W.dense(200 + m, cols)
        xs.append(torch.from_numpy(x).cuda())
        ys.append(torch.empty(len(pos) - 1, dtype=torch.float64, device="cuda"))
        refs.append(O.spmv(pos, crd, vals, x))
    plan = tg.SpmvBatch(mats, xs, ys, variants=[0] * len(mats))
    plan.run()
    torch.cuda.synchronize()
    for y, ref in zip(ys, refs):
        assert normwise(y.cpu().numpy(), ref) <= F64_TOL


def test_plan_reads_current_inputs(generated):
    """A plan computes from what its x arrays hold at run time (graph replays see updates)."""
    sub = generated[:8]
    mats = [tg.CsrMatrix.from_numpy(p, c, v, n) for p, c, v, n in sub]
    xs = [torch.from_numpy(W.dense(300 + m, n)).cuda() for m, (_, _, _, n) in enumerate(sub)]
    ys = [torch.empty(len(p) - 1, dtype=torch.float64, device="cuda") for p, _, _, _ in sub]
    plan = tg.SpmvBatch(mats, xs, ys)
    plan.run()
    for x in xs:
        x.mul_(-2.0)
    plan.run()
    torch.cuda.synchronize()
    for m, (pos, crd, vals, _) in enumerate(sub):
        ref = O.spmv(pos, crd, vals, xs[m].cpu().numpy())
        assert normwise(ys[m].cpu().numpy(), ref) <= F64_TOL


def test_double_float_out_of_range_tiles(generated):
    """Tiles with values outside the double-float range are recomputed natively in the batch."""
    sub = [list(t) for t in generated[:9]]
    for t in sub[::2]:
        t[2] = t[2].copy()
        t[2][: max(1, len(t[2]) // 4)] *= 2.0 ** 70
    ys, xs = _run([tuple(t) for t in sub], torch.float64, 0, [m % len(KINDS) for m in range(len(sub))])
    _check([tuple(t) for t in sub], ys, xs, F64_TOL)
