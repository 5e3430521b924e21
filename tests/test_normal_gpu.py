"""Normal-equation products A = K^T W K, b = K^T W dy (matrix_product,
retrieval.c:403-444; gradient, retrieval.c:573-577) on the GPU.

3xTF32 tensor-core path: |A - A_ref| <= 1e-5 sqrt(A_ii A_jj) (FP32 accumulation over m rows, m 2^-24; the
inputs are recovered to FP32 by 3xTF32); b within 1e-5 of sqrt(A_jj * dy^T W dy).
FP64 path: relative 1e-12 against numpy.
"""
import numpy as np
import pytest

from jurassic_gb300 import native, synth

pytestmark = pytest.mark.gpu


def _ref(K, w, dy):
    X = K * w[:, None]
    return X.T @ X, K.T @ (dy * w * w)


def _ctx():
    w = synth.config_limb_ega(n_rays=1)
    return native.Context(w.ctl)   # no tables needed for these products


@pytest.mark.parametrize("prec", [native.MIXED, native.FP64])
def test_normal_equations_uneven_batch(built_lib, prec):
    rng = np.random.default_rng(7)
    sizes = [(150, 405), (37, 64), (300, 129), (1, 1), (65, 63)]
    Ks = [rng.standard_normal((m, n)) * np.exp(rng.uniform(-3, 3, n))[None, :] for m, n in sizes]
    ws = [np.exp(rng.uniform(-1, 1, m)) for m, _ in sizes]
    dys = [rng.standard_normal(m) for m, _ in sizes]
    ctx = _ctx()
    As, bs = ctx.normal_equations(Ks, ws, dys, prec)
    for K, w, dy, A, b in zip(Ks, ws, dys, As, bs):
        Ar, br = _ref(K, w, dy)
        d = np.sqrt(np.diag(Ar))
        if prec == native.MIXED:
            assert np.max(np.abs(A - Ar) / np.outer(d, d)) <= 1e-5
            sdy = np.sqrt(np.sum((dy * w) ** 2))
            assert np.max(np.abs(b - br) / (d * sdy)) <= 1e-5
        else:
            assert np.max(np.abs(A - Ar) / np.outer(d, d)) <= 1e-12
            assert np.allclose(b, br, rtol=1e-10, atol=1e-12 * np.max(np.abs(br)))
        assert np.array_equal(A, A.T)


def test_normal_equations_many_tiles_per_sm(built_lib):
    """More output tiles than SMs: the persistent product kernel walks several
    tiles per CTA, so both tensor-memory accumulators are reused and the
    operand stages cycle across tiles of different chunk counts (m not a
    multiple of 16, n + 1 on and around multiples of 128).  Every problem
    meets the 3xTF32 bound, and a second call gives the same bits."""
    rng = np.random.default_rng(11)
    sizes = [(int(rng.integers(1, 121)), int(rng.choice([1, 127, 128, 255, 256])
                                            if i % 7 == 0 else rng.integers(1, 300)))
             for i in range(400)]
    Ks = [rng.standard_normal((m, n)) * np.exp(rng.uniform(-2, 2, n))[None, :] for m, n in sizes]
    ws = [np.exp(rng.uniform(-1, 1, m)) for m, _ in sizes]
    dys = [rng.standard_normal(m) for m, _ in sizes]
    tiles = sum(((n + 128) // 128) * ((n + 128) // 128 + 1) // 2 for _, n in sizes)
    assert tiles > 3 * 152
    ctx = _ctx()
    As, bs = ctx.normal_equations(Ks, ws, dys, native.MIXED)
    As2, bs2 = ctx.normal_equations(Ks, ws, dys, native.MIXED)
    for K, w, dy, A, b, A2, b2 in zip(Ks, ws, dys, As, bs, As2, bs2):
        Ar, br = _ref(K, w, dy)
        d = np.sqrt(np.diag(Ar))
        assert np.max(np.abs(A - Ar) / np.outer(d, d)) <= 1e-5
        sdy = np.sqrt(np.sum((dy * w) ** 2))
        assert np.max(np.abs(b - br) / (d * sdy)) <= 1e-5
        assert np.array_equal(A, A.T)
        assert np.array_equal(A, A2) and np.array_equal(b, b2)


def test_bounded_wait_gives_up_and_device_stays_usable(built_lib):
    """The tensor-core kernels' mbarrier waits are bounded: a wait for a phase
    that nothing completes gives up after about a second of the global timer
    and reports it (the kernel's error word turns into a status on the host);
    a phase that completes is seen at once; the device keeps working."""
    import ctypes as C
    L = native.load()
    to, sec = C.c_int(-1), C.c_double(-1.0)
    assert L.jgb_selftest_bounded_wait(0, 1, C.byref(to), C.byref(sec)) == 0
    assert to.value == 0 and sec.value < 0.01
    assert L.jgb_selftest_bounded_wait(0, 0, C.byref(to), C.byref(sec)) == 0
    assert to.value == 1 and 0.9 <= sec.value < 5.0
    rng = np.random.default_rng(3)
    K = [rng.standard_normal((40, 70))]
    w = [np.ones(40)]
    dy = [rng.standard_normal(40)]
    A, b = _ctx().normal_equations(K, w, dy, native.MIXED)
    Ar, br = _ref(K[0], w[0], dy[0])
    d = np.sqrt(np.diag(Ar))
    assert np.max(np.abs(A[0] - Ar) / np.outer(d, d)) <= 1e-5
