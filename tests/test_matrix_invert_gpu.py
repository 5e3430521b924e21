"""Batched matrix_invert (jgb_matrix_invert, retrieval.c:373-399) on the
GPU against the oracle's restatement: a ragged batch of diagonal matrices
(reciprocal diagonal, the lower triangle left alone), exponentially
correlated a-priori covariances and random symmetric positive-definite
matrices up to the Jacobian workload's n = 405, and matrices that are not
positive definite (status 1, left unchanged).  FP64 within 1e-10 of the
largest inverse entry (the factor's sums run in another order)."""
import numpy as np
import pytest

from jurassic_gb300 import native, synth
from oracle import oracle

pytestmark = pytest.mark.gpu


def _batch():
    rng = np.random.default_rng(17)
    mats = []
    d = np.diag(rng.uniform(0.5, 4.0, 9))
    d[5, 1] = 3.0                       # below the diagonal: still diagonal
    mats.append(d)
    for n, cz in ((1, 1.0), (31, 3.0), (101, 8.0), (405, 3.0)):
        z = np.sort(rng.uniform(0, 60, n))
        sig = rng.uniform(1, 3, n)
        mats.append(sig[:, None] * sig[None, :] * np.exp(-np.abs(z[:, None] - z[None, :]) / cz))
    for n in (2, 64, 300):
        b = rng.standard_normal((n, n))
        mats.append(b @ b.T / n + 0.5 * np.eye(n))
    mats.append(-np.eye(5) + 0.1)       # not positive definite
    mats.append(np.diag([1e-3, 2.0]) + np.diag([5.0], 1) + np.diag([5.0], -1))  # indefinite
    return mats


def test_matrix_invert_against_oracle(built_lib, built_oracle):
    w = synth.config_nadir(1, nd=2, nlev=11)
    ctx = native.Context(w.ctl, w.tables, w.filters)
    mats = _batch()
    inv, st = ctx.matrix_invert(mats)
    for k, (a, g, s) in enumerate(zip(mats, inv, st)):
        ref, ok = oracle.matrix_invert(a)
        assert (s == 0) == ok
        if not ok:
            assert np.array_equal(g, a)  # left as it was
            continue
        scale = np.max(np.abs(ref))
        assert np.max(np.abs(g - ref)) <= 1e-10 * scale
        if k > 0:  # the Cholesky branch symmetrises (the diagonal one does not)
            assert np.array_equal(g, g.T)
    # a diagonal matrix: exactly the reciprocals, nothing else touched
    d = mats[0]
    assert np.array_equal(np.diag(inv[0]), 1 / np.diag(d))
    assert inv[0][5, 1] == 3.0
    ctx.close()


def test_matrix_invert_without_tables(built_lib, built_oracle):
    # a context with only a control set (no tables, no source function)
    w = synth.config_nadir(1, nd=2, nlev=11)
    ctx = native.Context(w.ctl)
    mats = _batch()[1:4]
    inv, st = ctx.matrix_invert(mats)
    assert not np.any(st)
    for a, g in zip(mats, inv):
        ref, _ = oracle.matrix_invert(a)
        assert np.max(np.abs(g - ref)) <= 1e-10 * np.max(np.abs(ref))
    ctx.close()


def test_matrix_invert_rejects_bad_sizes(built_lib):
    w = synth.config_nadir(1, nd=2, nlev=11)
    ctx = native.Context(w.ctl, w.tables, w.filters)
    with pytest.raises(native.JurassicError):
        ctx.matrix_invert([np.zeros((0, 0))])
    ctx.close()
