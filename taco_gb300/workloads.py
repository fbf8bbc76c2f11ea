"""The synthetic sparse workloads the library is tested and measured on, as generator specs.

All matrices are CSR ({Dense,Sparse}, int32 pos/crd, sorted distinct columns per row) with
U(-1,1) values, produced by libtacogb_gen from a counter-based RNG (pure functions of the spec).

  spmv_small        65,536^2, row length uniform on [4,28] (~1.05M nnz)
  spmv_powerlaw     4,194,304^2, power-law rows: L = min(20000, max(1, round(c*K))),
                    K ~ Zipf(2) on [1,20000], c calibrated so E[L] = 24 (~1.0e8 nnz)
  spmv_banded       4,194,304^2, 32 distinct columns per row from the window [i-32, i+32)
  spmm_powerlaw     1,048,576^2, power-law rows with mean 32, max 10,000 (~3.4e7 nnz)
  spgemm_random     262,144^2, 8 nnz per row, uniform columns
  spgemm_poisson    5-point Laplacian on a 512x512 grid (diag 4, off-diagonal -1)
  batch matrix m    rows log-uniform in [256, 262,144], square, mean nnz/row from
                    {2,4,...,64}; uniform (lengths on [1, 2*mean-1]) / power-law / banded
                    (bandwidth 32) by m mod 3
"""
import numpy as np

from . import _native as N

UNIFORM, POWERLAW, BANDED, POISSON2D = 0, 1, 2, 3
SEED_BASE = 0x7AC0


def spec(rows, cols=None, kind=UNIFORM, len_lo=0, len_hi=0, mean=0.0, len_max=0, band=0,
         band_len=0, grid=0, seed=SEED_BASE):
    s = N.GenSpec()
    s.rows, s.cols, s.kind = rows, rows if cols is None else cols, kind
    s.len_lo, s.len_hi, s.mean, s.len_max = len_lo, len_hi, float(mean), len_max
    s.band, s.band_len, s.grid, s.seed = band, band_len, grid, seed
    return s


def spmv_small(seed=SEED_BASE + 1):
    return spec(65536, kind=UNIFORM, len_lo=4, len_hi=28, seed=seed)


def spmv_powerlaw(rows=4194304, seed=SEED_BASE + 2):
    return spec(rows, kind=POWERLAW, mean=24.0, len_max=min(20000, rows), seed=seed)


def spmv_banded(rows=4194304, seed=SEED_BASE + 2):
    return spec(rows, kind=BANDED, band=32, band_len=32, seed=seed)


def spmm_powerlaw(rows=1048576, seed=SEED_BASE + 3):
    return spec(rows, kind=POWERLAW, mean=32.0, len_max=min(10000, rows), seed=seed)


# SDDMM: the SpMM power-law matrix as the sampling pattern, J = 128 (taco's sddmmGPU width)
SDDMM_J = 128


def sddmm_powerlaw(rows=1048576, seed=SEED_BASE + 3):
    return spmm_powerlaw(rows, seed)


# Order-3 tensors for TTV / TTM / MTTKRP: nell-2's shape in FROSTT (12,092 x 9,184 x 28,818,
# 7.7e7 nonzeros) with synthetic structure: every i present, a power-law number of (i,k) fibers
# per i (mean 200) and of l per fiber (mean 32), values U(-1,1).
TENSOR3_DIMS = (12092, 9184, 28818)
MTTKRP_J = 32


def tensor3_powerlaw(dims=TENSOR3_DIMS, fib_mean=200.0, leaf_mean=32.0, seed=SEED_BASE + 5):
    """(dims, crd0, pos1, crd1, pos2, crd2, vals): a {Sparse,Sparse,Sparse} tensor."""
    s1 = spec(dims[0], cols=dims[1], kind=POWERLAW, mean=fib_mean, len_max=dims[1], seed=seed)
    pos1, crd1, _ = generate(s1)
    s2 = spec(len(crd1), cols=dims[2], kind=POWERLAW, mean=leaf_mean,
              len_max=min(dims[2], 4096), seed=seed + 1)
    pos2, crd2, vals = generate(s2)
    return (tuple(dims), np.arange(dims[0], dtype=np.int32), pos1, crd1, pos2, crd2, vals)


def spgemm_random(rows=262144, seed=SEED_BASE + 4):
    return spec(rows, kind=UNIFORM, len_lo=8, len_hi=8, seed=seed)


def spgemm_poisson(grid=512):
    return spec(grid * grid, kind=POISSON2D, grid=grid, seed=0)


def batch_spec(m, seed=SEED_BASE + 5, rows_lo=256, rows_hi=262144):
    s = N.GenSpec()
    N.gen().tacogb_gen_batch_spec(seed, m, rows_lo, rows_hi, s)
    return s


def generate(s, values=True):
    """(pos, crd, vals) numpy arrays for spec s."""
    g = N.gen()
    pos = np.empty(s.rows + 1, dtype=np.int32)
    nnz = g.tacogb_gen_pos(s, pos.ctypes.data)
    if nnz < 0:
        raise ValueError("matrix does not fit int32 positions")
    crd = np.empty(nnz, dtype=np.int32)
    vals = np.empty(nnz, dtype=np.float64) if values else None
    g.tacogb_gen_fill(s, pos.ctypes.data, crd.ctypes.data,
                      vals.ctypes.data if values else None)
    return pos, crd, vals


def dense(seed, count):
    """count U(-1,1) doubles."""
    out = np.empty(count, dtype=np.float64)
    N.gen().tacogb_gen_dense(seed, count, out.ctypes.data)
    return out


def powerlaw_scale(mean, kmax):
    return N.gen().tacogb_gen_powerlaw_scale(float(mean), kmax)
