"""The oracle's rank-revealing solve (qtzSolve, the restatement of the
reference's FactorQTZ used by the loop-closure multipliers and both
projections) against numpy's SVD-based minimum-norm least squares."""
import numpy as np
import pytest

from oracle import oracle as O

EPS = np.finfo(float).eps


def lstsq_min_norm(A, b, rank):
    U, s, Vt = np.linalg.svd(A, full_matrices=False)
    c = (U[:, :rank].T @ b) / s[:rank]
    return Vt[:rank].T @ c


@pytest.mark.parametrize("shape", [(6, 6), (12, 12), (3, 40), (9, 120)])
def test_full_rank_is_the_minimum_norm_solution(shape):
    rng = np.random.default_rng(sum(shape))
    A = rng.standard_normal(shape)
    b = rng.standard_normal(shape[0])
    x, r = O.qtz_solve(A, b, shape[0] * EPS ** 0.75)
    assert r == shape[0]
    ref = lstsq_min_norm(A, b, r)
    assert np.linalg.norm(x - ref) <= 1e-12 * np.linalg.norm(ref)


@pytest.mark.parametrize("square", [True, False])
def test_redundant_rows_drop_and_give_the_least_squares_minimum_norm(square):
    """A repeated closure repeats three rows; a second pinned point adds rows
    inside the span of the others. With a right side outside the range the
    least-squares minimum-norm solution is the reference's answer."""
    rng = np.random.default_rng(7 + square)
    n = 40
    G = rng.standard_normal((6, n))
    rows = np.vstack([G, G[:3], G[:2] + 0.5 * G[3:5]])  # 11 rows of rank 6
    A = rows @ np.diag(rng.uniform(0.5, 2.0, n)) @ rows.T if square else rows
    for consistent in (True, False):
        b = A @ rng.standard_normal(A.shape[1]) if consistent else rng.standard_normal(A.shape[0])
        tol = A.shape[0] * (EPS ** 0.75 if square else EPS ** 0.5)
        x, r = O.qtz_solve(A, b, tol)
        assert r == 6
        ref = lstsq_min_norm(A, b, 6)
        assert np.linalg.norm(x - ref) <= 1e-9 * np.linalg.norm(ref), (square, consistent)


def test_rank_follows_the_conditioning_tolerance():
    A = np.diag([1.0, 1e-3, 1e-7])
    b = np.ones(3)
    assert O.qtz_solve(A, b, 1e-9)[1] == 3
    assert O.qtz_solve(A, b, 1e-5)[1] == 2
    x, r = O.qtz_solve(A, b, 1e-2)
    assert r == 1 and np.allclose(x, [1, 0, 0])


def test_zero_matrix_has_rank_zero_and_a_zero_solution():
    x, r = O.qtz_solve(np.zeros((3, 5)), np.ones(3), 1e-8)
    assert r == 0 and not x.any()
