"""ORACLE — test infrastructure only (tests/ and bench.py's CPU legs).  The taco_gb300 product
never imports this module.

CPU restatements, in float64 numpy, of the batch autotuner's device code (taco_gb300/csrc/
tuner.cu): the sparsity features of a CSR matrix and the MLP cost model's forward pass and
gradient.  taco has no autotuner or cost model; these pin the project's own kernels.  The
gradient here is itself pinned by central finite differences in the tests.
"""
import numpy as np

F, H, K = 10, 32, 6
EXACT_BINS = 2048
LOG_BINS = 20 * 16
OW1 = 0
OB1 = OW1 + H * F
OW2 = OB1 + H
OB2 = OW2 + H * H
OW3 = OB2 + H
OB3 = OW3 + K * H
NPARAM = OB3 + K


def _len_bin(L):
    L = np.asarray(L, dtype=np.int64)
    out = L.copy()
    big = L >= EXACT_BINS
    if big.any():
        e = np.floor(np.log2(L[big])).astype(np.int64)
        # guard the float log2 at exact powers of two
        e = np.where((1 << e) > L[big], e - 1, e)
        e = np.where((1 << (e + 1)) <= L[big], e + 1, e)
        sub = (L[big] >> (e - 4)) & 15
        out[big] = EXACT_BINS + (np.minimum(e, 30) - 11) * 16 + sub
    return out


def features(pos, crd, cols):
    """The 10 features of batch_features for one CSR matrix (float64)."""
    pos = np.asarray(pos, dtype=np.int64)
    crd = np.asarray(crd, dtype=np.int64)
    n = len(pos) - 1
    L = np.diff(pos)
    S = float(pos[-1] - pos[0]) if n > 0 else 0.0
    mean = S / n if n > 0 else 0.0
    var = max(float((L * L).sum()) / n - mean * mean, 0.0) if n > 0 else 0.0
    g = 0.0
    if S > 0:
        b = _len_bin(L)
        cnt = np.bincount(b, minlength=EXACT_BINS + LOG_BINS).astype(np.float64)
        sums = np.bincount(b, weights=L.astype(np.float64), minlength=EXACT_BINS + LOG_BINS)
        r = np.concatenate([[0.0], np.cumsum(cnt)[:-1]])
        nz = cnt > 0
        g = float((sums[nz] * (2.0 * r[nz] + cnt[nz] - n)).sum()) / (n * S)
    rows = np.repeat(np.arange(n, dtype=np.int64), L)
    dist = np.abs(crd - rows)
    c = float(cols) if cols > 0 else 1.0
    return np.array([
        np.log2(n + 1.0), np.log2(S + 1.0), np.log2(mean + 1.0),
        np.sqrt(var) / mean if mean > 0 else 0.0, np.log2(float(L.max() if n else 0) + 1.0), g,
        float(dist.max()) / c if S > 0 else 0.0, float(dist.sum()) / S / c if S > 0 else 0.0,
        float((L == 0).sum()) / n if n > 0 else 0.0, np.log2(cols + 1.0)])


def unpack(params):
    p = np.asarray(params, dtype=np.float64)
    return (p[OW1:OB1].reshape(H, F), p[OB1:OW2], p[OW2:OB2].reshape(H, H), p[OB2:OW3],
            p[OW3:OB3].reshape(K, H), p[OB3:NPARAM])


def forward(params, norm, X):
    """Outputs (n x K) and the activations of the 10 -> 32 -> 32 -> K ReLU network."""
    W1, b1, W2, b2, W3, b3 = unpack(params)
    norm = np.asarray(norm, dtype=np.float64)
    x = (np.asarray(X, dtype=np.float64) - norm[:F]) / norm[F:]
    a1 = x @ W1.T + b1
    h1 = np.maximum(a1, 0.0)
    a2 = h1 @ W2.T + b2
    h2 = np.maximum(a2, 0.0)
    y = h2 @ W3.T + b3
    return y, (x, a1, h1, a2, h2)


def loss(params, norm, X, Y, M):
    y, _ = forward(params, norm, X)
    M = np.asarray(M, dtype=np.float64)
    return float((M * (y - Y) ** 2).sum() / M.sum())


def grad(params, norm, X, Y, M):
    """d loss / d params by reverse-mode differentiation, packed like the parameters."""
    W1, b1, W2, b2, W3, b3 = unpack(params)
    y, (x, a1, h1, a2, h2) = forward(params, norm, X)
    M = np.asarray(M, dtype=np.float64)
    d3 = 2.0 * M * (y - Y) / M.sum()
    d2 = (d3 @ W3) * (a2 > 0)
    d1 = (d2 @ W2) * (a1 > 0)
    g = np.empty(NPARAM)
    g[OW1:OB1] = (d1.T @ x).ravel()
    g[OB1:OW2] = d1.sum(0)
    g[OW2:OB2] = (d2.T @ h1).ravel()
    g[OB2:OW3] = d2.sum(0)
    g[OW3:OB3] = (d3.T @ h2).ravel()
    g[OB3:NPARAM] = d3.sum(0)
    return g


def finite_difference(params, norm, X, Y, M, idx, h=1e-6):
    """Central differences of the loss for the parameter indices idx."""
    p = np.asarray(params, dtype=np.float64).copy()
    out = []
    for i in idx:
        keep = p[i]
        p[i] = keep + h
        lp = loss(p, norm, X, Y, M)
        p[i] = keep - h
        lm = loss(p, norm, X, Y, M)
        p[i] = keep
        out.append((lp - lm) / (2 * h))
    return np.array(out)
