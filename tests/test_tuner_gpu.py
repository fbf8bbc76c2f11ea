"""The autotuner's GPU kernels against the CPU oracle (oracle/tuner_oracle.py): sparsity features,
the cost model's forward pass and gradient, deterministic training, the exhaustive autotuner,
learned selection, and what the trained model gains over the method without it.

Bars: features within float32 rounding of the float64 oracle (relative 1e-6); forward pass and
gradient within 1e-5 and 1e-4 normwise of the float64 oracle (float32 kernels, 1,606
parameters; a ReLU whose input rounds across zero differently in float32 moves one sample)."""
import ctypes
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import taco_gb300 as tg  # noqa: E402
from oracle import oracle as O  # noqa: E402
from oracle import tuner_oracle as TO  # noqa: E402
from taco_gb300 import autotune as AT  # noqa: E402
from taco_gb300 import workloads as W  # noqa: E402
from tests.helpers import normwise  # noqa: E402

pytestmark = pytest.mark.gpu


def _matrices():
    rng = np.random.default_rng(17)
    out = []
    out.append((np.zeros(1, np.int32), np.zeros(0, np.int32), 5))
    out.append((np.zeros(70, np.int32), np.zeros(0, np.int32), 9))
    lens = rng.integers(0, 40, 3000)
    lens[[5, 700, 2500]] = [2047, 2048, 70000]  # both sides of the exact/log bin edge
    pos = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    crd = np.concatenate([np.sort(rng.choice(80000, n, replace=False)) for n in lens])
    out.append((pos, crd.astype(np.int32), 80000))
    for m in range(12):
        s = W.batch_spec(m, rows_hi=30000)
        p, c, _ = W.generate(s, values=False)
        out.append((p, c, s.cols))
    return out


def _csr(pos, crd, cols):
    vals = np.zeros(len(crd))
    return tg.CsrMatrix.from_numpy(pos, crd, vals, cols)


def test_features_match_oracle():
    mats_np = _matrices()
    mats = [_csr(*t) for t in mats_np]
    got = AT.features(mats)
    for m, (pos, crd, cols) in enumerate(mats_np):
        ref = TO.features(pos, crd, cols).astype(np.float32).astype(np.float64)
        np.testing.assert_allclose(got[m], ref, rtol=1e-6, atol=1e-7, err_msg=str(m))


def _problem(n, seed):
    rng = np.random.default_rng(seed)
    X = rng.normal(2.0, 3.0, size=(n, TO.F)).astype(np.float32)
    Y = rng.normal(size=(n, TO.K)).astype(np.float32)
    M = (rng.random((n, TO.K)) > 0.15).astype(np.float32)
    model = AT.CostModel.initial(X, seed=seed)
    return X, Y, M, model


@pytest.mark.parametrize("n", [1, 127, 300, 5000])
def test_forward_and_gradient_match_oracle(n):
    X, Y, M, model = _problem(n, n)
    M[0, :] = 1.0
    pred, kinds = model.predict(X)
    ref = TO.forward(model.params, model.norm, X)[0]
    assert normwise(pred.astype(np.float64), ref) <= 1e-5
    assert np.array_equal(kinds, np.argmin(pred, axis=1))
    dev = [torch.from_numpy(a).cuda() for a in (model.params, model.norm, X, Y, M)]
    g = torch.empty(TO.NPARAM, dtype=torch.float32, device="cuda")
    loss = torch.empty(1, dtype=torch.float32, device="cuda")
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    tg.check(tg.lib().tacogb_mlp_grad(*[d.data_ptr() for d in dev], n, g.data_ptr(),
                                      loss.data_ptr(), st), "tacogb_mlp_grad")
    gref = TO.grad(model.params, model.norm, X, Y, M)
    assert normwise(g.cpu().double().numpy(), gref) <= 1e-4
    assert abs(float(loss) - TO.loss(model.params, model.norm, X, Y, M)) <= 1e-5 * (
        1 + TO.loss(model.params, model.norm, X, Y, M))


def test_training_is_deterministic_and_descends():
    X, Y, M, model = _problem(2000, 3)
    Y = (X[:, :TO.K] * 0.3 + np.sin(X[:, 1:2])).astype(np.float32)  # learnable targets
    m1 = AT.CostModel(model.params.copy(), model.norm)
    m2 = AT.CostModel(model.params.copy(), model.norm)
    l1 = m1.fit(X, Y, M, steps=400, lr=3e-3)
    l2 = m2.fit(X, Y, M, steps=400, lr=3e-3)
    assert np.array_equal(m1.params, m2.params) and np.array_equal(l1, l2)
    assert l1[-1] < 0.2 * l1[0]


@pytest.fixture(scope="module")
def small_batch():
    mats, xs, ys, refs = [], [], [], []
    for m in range(40):
        s = W.batch_spec(m, seed=99, rows_hi=40000)
        pos, crd, vals = W.generate(s)
        mats.append(tg.CsrMatrix.from_numpy(pos, crd, vals, s.cols, dtype=torch.float32))
        x = W.dense(500 + m, s.cols)
        xs.append(torch.from_numpy(x).float().cuda())
        ys.append(torch.empty(s.rows, dtype=torch.float32, device="cuda"))
        refs.append(O.spmv(pos, crd, vals, x))
    return mats, xs, ys, refs


def test_exhaustive_autotuner(small_batch):
    mats, xs, ys, refs = small_batch
    kinds, cycles = AT.exhaustive(mats, xs, ys, reps=2)
    assert cycles.shape == (len(mats), TO.K) and np.all(cycles > 0)
    assert np.array_equal(kinds, np.argmin(cycles, axis=1))
    assert AT.regret(cycles, kinds) == 0.0
    plan = tg.SpmvBatch(mats, xs, ys, variants=kinds)
    plan.run()
    torch.cuda.synchronize()
    for y, ref in zip(ys, refs):  # the tuned plan computes the same products
        assert normwise(y.double().cpu().numpy(), ref) <= 1e-6


def test_learned_select_matches_features_and_predict(small_batch):
    mats = small_batch[0]
    X = AT.features(mats)
    model = AT.CostModel.initial(X, seed=4)
    _, kinds = model.predict(X)
    assert np.array_equal(AT.learned_select(model, mats), kinds)


@pytest.mark.skipif(not os.path.exists(AT.DB_PATH), reason="no timing database")
def test_model_gains_over_static_choice():
    """Trained on the committed timing database (GPU training kernels), the model's choices on
    held-out matrices cost less than the best single kind, and stay near the exhaustive
    autotuner's per-matrix optimum."""
    z = np.load(AT.DB_PATH)
    model, losses, te = AT.train_from_db(z, steps=3000)
    assert losses[-1] < 0.25 * losses[0]
    _, kinds = model.predict(z["features"][te])
    cyc = z["cycles"][te]
    k, r_static = AT.static_best(cyc)
    r = AT.regret(cyc, kinds)
    print("held-out regret: learned %.4f, best single kind %s %.4f" % (
        r, tg.batch_variants()[k], r_static))
    assert r < r_static
    assert r <= 0.10
