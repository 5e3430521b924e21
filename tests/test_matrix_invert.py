"""matrix_invert (retrieval.c:373-399) in the oracle (CPU): the reciprocal
diagonal where every element right of the diagonal is zero, else the
Cholesky inverse; a matrix that is not positive definite is reported.
Checked against numpy's inverse."""
import numpy as np

from oracle import oracle


def _spd(rng, n):
    b = rng.standard_normal((n, n))
    return b @ b.T / n + np.eye(n)


def test_oracle_inverse_of_spd_matrices():
    rng = np.random.default_rng(3)
    for n in (1, 2, 7, 60):
        a = _spd(rng, n)
        inv, ok = oracle.matrix_invert(a)
        ref = np.linalg.inv(a)
        assert ok
        assert np.max(np.abs(inv - ref)) <= 1e-12 * np.max(np.abs(ref))
        assert np.array_equal(inv, inv.T)  # symmetrised


def test_oracle_diagonal_rule():
    # only elements right of the diagonal decide (retrieval.c:379-385): a
    # lower triangle is ignored and the diagonal is inverted elementwise
    a = np.diag([2.0, -4.0, 0.5])
    a[2, 0] = 7.0
    inv, ok = oracle.matrix_invert(a)
    assert ok
    assert np.array_equal(np.diag(inv), [0.5, -0.25, 2.0])
    assert inv[2, 0] == 7.0


def test_oracle_not_positive_definite():
    a = -np.eye(4) + 0.1
    _, ok = oracle.matrix_invert(a)
    assert not ok
