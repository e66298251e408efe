"""The algebra behind two accept paths, checked in numpy on the CPU.

1. FP64 accepts of more than 32 edges take W = D K^-1 X from an explicit
   inverse plus one refinement step, W = W0 - Vneg (X - K D W0) with
   Vneg = -D K^-1 and W0 = -Vneg X: an inverse carrying a relative error e
   leaves W0 off by about e and W by about cond(K) e^2 plus rounding.
2. The deferred complex64 form reads T_true = T - U Vt^T with U and Vt stored
   row by row (N x rcap, rank index fastest): the rows and the columns s of
   T_true formed as dense blocks equal the elementwise reads."""
import numpy as np


def _rand_c(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def test_refined_w_recovers_solve_accuracy():
    rng = np.random.default_rng(3)
    k, n = 48, 300
    U_, _ = np.linalg.qr(_rand_c(rng, k, k))
    V_, _ = np.linalg.qr(_rand_c(rng, k, k))
    K = U_ @ np.diag(np.logspace(0, -3, k)) @ V_  # cond(K) = 1e3
    d = rng.choice([-1.0, 1.0], size=k)
    D = np.diag(d)
    X = _rand_c(rng, k, n)
    W_true = D @ np.linalg.solve(K, X)
    Kinv = np.linalg.inv(K)
    Kinv_bad = Kinv * (1 + 1e-9 * _rand_c(rng, k, k))  # an inverse with a relative error of 1e-9
    Vneg = -D @ Kinv_bad
    W0 = -Vneg @ X
    W1 = W0 - Vneg @ (X - (K @ D) @ W0)
    scale = np.abs(W_true).max()
    e0 = np.abs(W0 - W_true).max() / scale
    e1 = np.abs(W1 - W_true).max() / scale
    assert e0 > 1e-10
    assert e1 < 1e-4 * e0 and e1 < 1e-12


def test_pending_blocks_equal_elementwise_reads():
    rng = np.random.default_rng(5)
    n, rcap, rp, k = 200, 24, 17, 9
    T = _rand_c(rng, n, n).astype(np.complex64)
    U = _rand_c(rng, n, rcap).astype(np.complex64)   # row i: U[i, :rcap]
    Vt = _rand_c(rng, n, rcap).astype(np.complex64)  # row j: Vt[j, :rcap]
    s = np.sort(rng.choice(n, size=k, replace=False))

    def t_true(i, j):  # the view's read: T[i, j] - sum_q U[i, q] Vt[j, q]
        return T[i, j].astype(np.complex128) - np.sum(U[i, :rp].astype(np.complex128) *
                                                      Vt[j, :rp].astype(np.complex128))

    rows = T[s, :].astype(np.complex128) - U[s, :rp].astype(np.complex128) @ Vt[:, :rp].T.astype(np.complex128)
    cols = T[:, s].astype(np.complex128) - U[:, :rp].astype(np.complex128) @ Vt[s, :rp].T.astype(np.complex128)
    for r, i in enumerate(s):
        for j in range(0, n, 37):
            assert abs(rows[r, j] - t_true(i, j)) <= 1e-12 * (1 + abs(rows[r, j]))
    for c, j in enumerate(s):
        for i in range(0, n, 41):
            assert abs(cols[i, c] - t_true(i, j)) <= 1e-12 * (1 + abs(cols[i, c]))
