"""Batch autotuning: the exhaustive autotuner, the timing database it produces, and the MLP cost
model trained on that database with the library's own GPU kernels.

    features(mats)                 sparsity features (tacogb_batch_features, on the GPU)
    exhaustive(mats, xs, ys)       per-matrix cycles of every work-unit kind and the argmin
                                   (tacogb_batch_autotune: the labels the model is scored
                                   against, and the fallback)
    CostModel                      10 -> 32 -> 32 -> 6 ReLU network; fit() runs
                                   tacogb_mlp_train (forward, backward and Adam kernels),
                                   predict() tacogb_mlp_predict
    learned_select(model, mats)    tacogb_batch_select: features + the model's argmin
    regret(cycles, kinds)          sum of chosen cycles over the sum of the per-matrix best - 1

The database (collect()) holds, for matrices drawn from the batch generator with its own seed,
the features and the minimum over repeated runs of every kind's SM cycles inside a full-batch
persistent launch.  The model's target is log2(cycles / (rows + nnz + 1)) per kind.

Run `python -m taco_gb300.autotune collect --count N --out FILE` on a GPU to (re)build a
database and `python -m taco_gb300.autotune train --db FILE --out MODEL` to fit a model.
"""
import argparse
import ctypes
import os
import time

import numpy as np

from . import _native as N

F, H, K = 10, 32, 6
DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")
DB_PATH = os.path.join(DATA, "batch_timings_f32c.npz")
MODEL_PATH = os.path.join(DATA, "batch_mlp.npz")
DB_SEED = 0x7AC0 + 6  # the benchmark batch uses SEED_BASE + 5


def _stream(stream):
    from . import _stream_ptr
    return _stream_ptr(stream)


def _csrs(mats):
    return (N.Csr * len(mats))(*[A.as_csr() for A in mats])


def features(mats, stream=None):
    out = np.empty((len(mats), F), dtype=np.float32)
    N.check(N.lib().tacogb_batch_features(len(mats), _csrs(mats), out.ctypes.data,
                                          _stream(stream)), "tacogb_batch_features")
    return out


def exhaustive(mats, xs, ys, precision=0, reps=3, stream=None):
    n = len(mats)
    kinds = np.empty(n, dtype=np.int32)
    cycles = np.empty((n, K), dtype=np.int64)
    xp = (ctypes.c_void_p * n)(*[x.data_ptr() for x in xs])
    yp = (ctypes.c_void_p * n)(*[y.data_ptr() for y in ys])
    N.check(N.lib().tacogb_batch_autotune(n, _csrs(mats), xp, yp, precision, reps,
                                          kinds.ctypes.data, cycles.ctypes.data,
                                          _stream(stream)), "tacogb_batch_autotune")
    return kinds, cycles


def targets(cycles, rows, nnz):
    """(Y, M): log2 cycles per (row + nonzero) and the mask of measured entries."""
    c = np.asarray(cycles, dtype=np.float64)
    items = (np.asarray(rows, dtype=np.float64) + np.asarray(nnz, dtype=np.float64) + 1.0)[:, None]
    M = (c > 0).astype(np.float32)
    Y = np.where(c > 0, np.log2(np.maximum(c, 1.0) / items), 0.0).astype(np.float32)
    return Y, M


def regret(cycles, kinds):
    c = np.asarray(cycles, dtype=np.float64)
    chosen = c[np.arange(len(c)), np.asarray(kinds)].sum()
    return float(chosen / c.min(axis=1).sum() - 1.0)


def static_best(cycles):
    """The single kind with the lowest total cycles over all matrices, and its regret."""
    c = np.asarray(cycles, dtype=np.float64)
    k = int(np.argmin(c.sum(axis=0)))
    return k, regret(c, np.full(len(c), k))


class CostModel:
    def __init__(self, params, norm):
        self.params = np.asarray(params, dtype=np.float32)
        self.norm = np.asarray(norm, dtype=np.float32)
        assert self.params.size == N.lib().tacogb_mlp_param_count()

    @classmethod
    def initial(cls, X, seed=0):
        """He-initialised weights, zero biases; norm from the features X."""
        rng = np.random.default_rng(seed)
        p = []
        for fan_out, fan_in in ((H, F), (H, H), (K, H)):
            p.append(rng.normal(0.0, np.sqrt(2.0 / fan_in), fan_out * fan_in))
            p.append(np.zeros(fan_out))
        X = np.asarray(X, dtype=np.float64)
        sd = X.std(axis=0)
        norm = np.concatenate([X.mean(axis=0), np.where(sd > 1e-12, sd, 1.0)])
        return cls(np.concatenate(p), norm)

    def _dev(self, torch):
        return (torch.from_numpy(self.params).cuda(), torch.from_numpy(self.norm).cuda())

    def fit(self, X, Y, M, steps=3000, lr=3e-3, stream=None):
        """Full-batch Adam on the GPU; returns the loss before every step."""
        import torch
        P, nm = self._dev(torch)
        dX, dY, dM = (torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()
                      for a in (X, Y, M))
        state = torch.zeros(2 * P.numel(), dtype=torch.float32, device="cuda")
        losses = torch.empty(max(steps, 1), dtype=torch.float32, device="cuda")
        N.check(N.lib().tacogb_mlp_train(P.data_ptr(), nm.data_ptr(), dX.data_ptr(),
                                         dY.data_ptr(), dM.data_ptr(), len(X), steps, 0,
                                         ctypes.c_float(lr), state.data_ptr(), losses.data_ptr(),
                                         _stream(stream)), "tacogb_mlp_train")
        torch.cuda.synchronize()
        self.params = P.cpu().numpy()
        return losses[:steps].cpu().numpy()

    def predict(self, X, stream=None):
        import torch
        P, nm = self._dev(torch)
        dX = torch.from_numpy(np.ascontiguousarray(X, dtype=np.float32)).cuda()
        pred = torch.empty(len(X), K, dtype=torch.float32, device="cuda")
        kinds = torch.empty(len(X), dtype=torch.int32, device="cuda")
        N.check(N.lib().tacogb_mlp_predict(P.data_ptr(), nm.data_ptr(), dX.data_ptr(), len(X),
                                           pred.data_ptr(), kinds.data_ptr(), _stream(stream)),
                "tacogb_mlp_predict")
        torch.cuda.synchronize()
        return pred.cpu().numpy(), kinds.cpu().numpy()

    def save(self, path, **meta):
        np.savez(path, params=self.params, norm=self.norm, **meta)

    @classmethod
    def load(cls, path):
        z = np.load(path)
        return cls(z["params"], z["norm"])


def load_model(path=MODEL_PATH):
    return CostModel.load(path)


def learned_select(model, mats, stream=None):
    import torch
    P, nm = model._dev(torch)
    kinds = np.empty(len(mats), dtype=np.int32)
    N.check(N.lib().tacogb_batch_select(len(mats), _csrs(mats), P.data_ptr(), nm.data_ptr(),
                                        kinds.ctypes.data, _stream(stream)), "tacogb_batch_select")
    return kinds


def exhaustive_select(mats, xs, ys, precision=0, reps=3):
    return exhaustive(mats, xs, ys, precision, reps)


# ------------------------------------------------------------------------ database ------

def collect(count, seed=DB_SEED, group_nnz=1.2e9, reps=3, log=print):
    """Features and per-kind cycles of `count` generated matrices (FP32 values, compensated
    accumulation), measured in groups of about group_nnz nonzeros per persistent launch."""
    import torch
    import taco_gb300 as tg
    from . import workloads as W
    feats, cycles, rows, nnz = [], [], [], []
    m = 0
    t0 = time.time()
    while m < count:
        mats, xs, ys, tot = [], [], [], 0
        while m < count and tot < group_nnz:
            s = W.batch_spec(m, seed=seed)
            pos, crd, vals = W.generate(s)
            mats.append(tg.CsrMatrix.from_numpy(pos, crd, vals, s.cols, dtype=torch.float32))
            xs.append(torch.rand(s.cols, device="cuda") * 2 - 1)
            ys.append(torch.empty(s.rows, device="cuda"))
            rows.append(s.rows)
            nnz.append(len(crd))
            tot += len(crd)
            m += 1
        feats.append(features(mats))
        _, c = exhaustive(mats, xs, ys, precision=0, reps=reps)
        cycles.append(c)
        log("collected %d / %d matrices (%.0f s)" % (m, count, time.time() - t0))
        del mats, xs, ys
        torch.cuda.empty_cache()
    return (np.concatenate(feats), np.concatenate(cycles), np.array(rows, np.int64),
            np.array(nnz, np.int64))


def split(n, test_frac=0.2, seed=1):
    idx = np.random.default_rng(seed).permutation(n)
    nt = int(n * test_frac)
    return idx[nt:], idx[:nt]


def train_from_db(db, steps=3000, lr=3e-3, seed=0):
    """Trains on the database's training split; returns (model, losses, test indices)."""
    z = np.load(db) if isinstance(db, str) else db
    Y, M = targets(z["cycles"], z["rows"], z["nnz"])
    tr, te = split(len(Y))
    model = CostModel.initial(z["features"][tr], seed=seed)
    losses = model.fit(z["features"][tr], Y[tr], M[tr], steps=steps, lr=lr)
    return model, losses, te


def main():
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    c = sub.add_parser("collect")
    c.add_argument("--count", type=int, default=20000)
    c.add_argument("--out", default=DB_PATH)
    c.add_argument("--reps", type=int, default=3)
    t = sub.add_parser("train")
    t.add_argument("--db", default=DB_PATH)
    t.add_argument("--out", default=MODEL_PATH)
    t.add_argument("--steps", type=int, default=3000)
    a = ap.parse_args()
    if a.cmd == "collect":
        import torch
        f, cyc, rows, nnz = collect(a.count, reps=a.reps)
        np.savez_compressed(a.out, features=f, cycles=cyc, rows=rows, nnz=nnz, seed=DB_SEED,
                            device=torch.cuda.get_device_name(), reps=a.reps)
        print("wrote", a.out, f.shape)
    else:
        z = np.load(a.db)
        model, losses, te = train_from_db(z, steps=a.steps)
        pred, kinds = model.predict(z["features"][te])
        cyc = z["cycles"][te]
        k, r_static = static_best(cyc)
        r = regret(cyc, kinds)
        model.save(a.out, test_regret=r, static_kind=k, static_regret=r_static,
                   final_loss=losses[-1])
        print("loss %.4f -> %.4f; held-out regret %.4f (best single kind %d: %.4f)" % (
            losses[0], losses[-1], r, k, r_static))


if __name__ == "__main__":
    main()
