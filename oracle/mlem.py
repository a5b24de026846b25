"""FP64 restatement of the reference's MLEM loop (main.m:154-176).

TEST INFRASTRUCTURE ONLY: the checker of the CUDA MLEM.  Only the tests, the
smoke check and bench.py's CPU-baseline leg use it.
"""
import numpy as np


def mlem_matrix(A, y, c, x0, iters):
    """A: [rays, K] (the Amatrix rows), y, c: [rays], x0: [K].

    x <- x .* (A' (y ./ (A x + c + 1e-20))) ./ (sum(A,1)' + 1e-7)   (main.m:162)
    x(~isfinite(x)) = 0                                              (main.m:163)
    x(x < 0) = 0                                                     (main.m:176)
    """
    A = np.asarray(A, np.float64)
    y = np.asarray(y, np.float64)
    c = np.asarray(c, np.float64)
    x = np.array(x0, np.float64)
    sens = A.sum(0) + 1e-7
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        for _ in range(iters):
            x = x * (A.T @ (y / (A @ x + c + 1e-20))) / sens
            x[~np.isfinite(x)] = 0.0
            x[x < 0] = 0.0
    return x
