"""The tensor-core FP64 Gram product (tcgen05 MMA on exact 7-bit digit slices, ozaki.cu) against
FP64 references: numpy's X^T Y and the library's FP64 CUDA-core kernel, through the C ABI
(fem2d_block_gram_device). The slicing error is bounded per 128-row chunk by 2^-49 times
rows x max|x_i| x max|y_j| of the chunk; the tests hold the result to that bound (plus the reference's
own rounding), and to 1e-13 of |X|^T |Y| for well-scaled data."""
import numpy as np
import pytest

import fem_2d_gb300 as fg

pytestmark = pytest.mark.gpu


def _chunk_bound(X, Y, chunk=128):
    n = X.shape[0]
    bound = np.zeros((X.shape[1], Y.shape[1]))
    for c0 in range(0, n, chunk):
        xs, ys = X[c0:c0 + chunk], Y[c0:c0 + chunk]
        bound += len(xs) * np.outer(np.max(np.abs(xs), axis=0), np.max(np.abs(ys), axis=0))
    return 2.0 ** -49 * bound


def _gram(ctx, method, X, Y):
    torch = pytest.importorskip("torch")
    dx = torch.from_numpy(np.ascontiguousarray(X)).cuda()
    dy = torch.from_numpy(np.ascontiguousarray(Y)).cuda()
    dc = torch.full((X.shape[1], Y.shape[1]), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    fg.block_gram_device(ctx, method, X.shape[0], dx.data_ptr(), X.shape[1], X.shape[1], dy.data_ptr(), Y.shape[1],
                         Y.shape[1], dc.data_ptr())
    return dc.cpu().numpy()


@pytest.fixture(scope="module")
def ctx():
    return fg.Context(0)


@pytest.mark.parametrize("n,a,b", [(1, 1, 1), (129, 5, 3), (100003, 150, 30), (20000, 150, 150), (4096, 300, 40)])
def test_tensor_gram_gaussian(ctx, n, a, b):
    rng = np.random.default_rng(n + a + b)
    X = rng.standard_normal((n, a))
    Y = rng.standard_normal((n, b))
    ref = X.T @ Y
    absref = np.abs(X).T @ np.abs(Y)
    C0 = _gram(ctx, fg.GRAM_TENSOR, X, Y)
    C1 = _gram(ctx, fg.GRAM_FP64, X, Y)
    assert np.all(np.isfinite(C0))
    assert np.max(np.abs(C0 - ref) / absref) < 1e-13
    assert np.max(np.abs(C1 - ref) / absref) < 1e-13
    assert np.all(np.abs(C0 - ref) <= _chunk_bound(X, Y) + 1e-15 * n * absref)
    # deterministic: the same call gives the same bits
    assert np.array_equal(C0, _gram(ctx, fg.GRAM_TENSOR, X, Y))


def test_tensor_gram_wide_dynamic_range(ctx):
    """Rows scaled over 30 orders of magnitude, exact zeros and negative values: the per-chunk column
    scaling keeps the error within the chunk bound."""
    rng = np.random.default_rng(5)
    n, a, b = 50000, 64, 24
    X = rng.standard_normal((n, a)) * 10.0 ** rng.uniform(-15, 15, size=(n, 1))
    Y = rng.standard_normal((n, b)) * 10.0 ** rng.uniform(-15, 15, size=(n, 1))
    X[::7, 3] = 0.0
    Y[:, 5] = 0.0
    ref = X.T @ Y
    C0 = _gram(ctx, fg.GRAM_TENSOR, X, Y)
    bound = _chunk_bound(X, Y) + 1e-15 * n * (np.abs(X).T @ np.abs(Y))
    assert np.all(np.abs(C0 - ref) <= bound)
    assert np.all(C0[:, 5] == 0.0)


def test_tensor_gram_symmetric_products(ctx):
    """X^T X (the B-orthogonalisation Gram form) is symmetric to rounding and positive on the diagonal."""
    rng = np.random.default_rng(11)
    X = rng.standard_normal((30000, 40))
    G = _gram(ctx, fg.GRAM_TENSOR, X, X)
    assert np.max(np.abs(G - G.T)) <= 1e-13 * np.max(np.abs(G))
    d = np.sum(X * X, axis=0)
    assert np.all(np.abs(np.diag(G) - d) <= np.diag(_chunk_bound(X, X)) + 1e-15 * X.shape[0] * d)


def _gemm(ctx, method, X, C, Z0, alpha, beta):
    torch = pytest.importorskip("torch")
    dx = torch.from_numpy(np.ascontiguousarray(X)).cuda()
    dc = torch.from_numpy(np.ascontiguousarray(C)).cuda()
    dz = torch.from_numpy(np.ascontiguousarray(Z0)).cuda()
    torch.cuda.synchronize()
    n, a = X.shape
    b = C.shape[1]
    fg.block_gemm_device(ctx, method, n, dx.data_ptr(), a, a, dc.data_ptr(), b, alpha, beta, dz.data_ptr(), b)
    return dz.cpu().numpy()


@pytest.mark.parametrize("n,a,b,beta", [(1, 1, 1, 0.0), (300, 7, 5, 1.0), (100003, 150, 30, 1.0),
                                        (20000, 256, 32, 0.0), (50000, 129, 17, -0.5)])
def test_tensor_block_update(ctx, n, a, b, beta):
    """Z = beta Z + alpha X C: the per-row / per-column slicing bound is 2^-49 a max|x_i| max|c_j|."""
    rng = np.random.default_rng(n + 3 * a + b)
    X = rng.standard_normal((n, a)) * 10.0 ** rng.uniform(-3, 3, size=(n, 1))
    C = rng.standard_normal((a, b))
    Z0 = rng.standard_normal((n, b))
    alpha = -1.0
    ref = beta * Z0 + alpha * (X @ C)
    Zt = _gemm(ctx, fg.GRAM_TENSOR, X, C, Z0, alpha, beta)
    Zf = _gemm(ctx, fg.GRAM_FP64, X, C, Z0, alpha, beta)
    bound = 2.0 ** -49 * a * np.outer(np.max(np.abs(X), axis=1), np.max(np.abs(C), axis=0)) \
        + 1e-15 * (abs(beta) * np.abs(Z0) + a * (np.abs(X) @ np.abs(C)))
    assert np.all(np.abs(Zt - ref) <= bound)
    assert np.all(np.abs(Zf - ref) <= bound)


@pytest.mark.parametrize("which", [0, 1])
def test_tensor_spmm_against_fp64(ctx, which):
    """Y = c M X for M = A or B of a full-form GEP (row runs of 1..64 rows, 128-column chunks), against
    the FP64 product: within 2^-48 x (per chunk) max|m_row| max|x_col| x 128, i.e. at FP64 rounding
    level of |M| |X| for well-scaled columns; checked against |M| |X| at 1e-13."""
    torch = pytest.importorskip("torch")
    from fem_2d_gb300 import configs

    w = configs.full_scale(seed=1, nx=8, ny=4, rounds=2, fraction=0.44)
    d = fg.Domain.from_mesh(configs.build_mesh(w))
    g = fg.galerkin_sample_gep_hcurl(fg.HierPoly, fg.CurlCurl, fg.L2Inner, d, [10, 10], ctx=ctx)
    A, B = g.scipy()
    M = A if which == 0 else B
    n = g.dimension
    rng = np.random.default_rng(which)
    for nb in (1, 17, 32):
        X = rng.standard_normal((n, nb))
        dx = torch.from_numpy(X).cuda()
        dy = torch.full((n, nb), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        g.spmm_tensor_device(which, -2.0, dx.data_ptr(), nb, nb, dy.data_ptr(), nb)
        Y = dy.cpu().numpy()
        ref = -2.0 * (M @ X)
        absref = 2.0 * (abs(M) @ np.abs(X))
        assert np.all(np.isfinite(Y))
        assert np.max(np.abs(Y - ref) / np.maximum(absref, 1e-300)) < 1e-13


def test_mma_issue_cost(ctx):
    """The measured issue cost of tcgen05.mma (M = 128, K = 16) is positive, does not fall as N grows,
    and an MMA with N = 256 does at least twice the work per ns of one with N = 32 (the shapes of the
    tensor-core kernels rest on this)."""
    c = {n: ctx.mma_ns(n) for n in (32, 64, 256)}
    assert all(v > 0 for v in c.values())
    assert c[256] >= 0.9 * c[32]
    assert (256 / c[256]) >= 2.0 * (32 / c[32])
    with pytest.raises(fg.Fem2dError):
        ctx.mma_ns(24)
