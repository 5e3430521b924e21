"""Host threads sharing one context on the GPU.

The reference's kernel() runs formod from OpenMP threads at once
(jurassic.c:4036).  Every entry point of a context holds the context's lock,
so calls from several host threads on one context run one after another:
each thread's forward models (both precisions, host buffers with their
pipelined chunk copies) and normal equations equal the same calls made alone,
bit for bit.
"""
import threading

import numpy as np
import pytest

from jurassic_gb300 import native, synth

pytestmark = pytest.mark.gpu


def test_threads_share_a_context(built_lib):
    w = synth.config_nadir(300, nd=24, nlev=61, ztop=60.0, emitters=("CO2", "H2O"))
    ctx = native.Context(w.ctl, w.tables, w.filters)
    ref = {prec: ctx.formod_batch(w.batch.fresh_outputs(), prec)
           for prec in (native.FP64, native.MIXED)}
    rng = np.random.default_rng(5)
    Ks = [rng.standard_normal((60, 90)) for _ in range(6)]
    ws = [np.exp(rng.uniform(-1, 1, 60)) for _ in range(6)]
    dys = [rng.standard_normal(60) for _ in range(6)]
    ne_ref = ctx.normal_equations(Ks, ws, dys, native.MIXED)

    out, errors = [], []

    def work(i):
        try:
            for rep in range(3):
                if i == 5:
                    out.append(("ne", ctx.normal_equations(Ks, ws, dys, native.MIXED)))
                else:
                    prec = (native.FP64, native.MIXED)[(i + rep) % 2]
                    out.append((prec, ctx.formod_batch(w.batch.fresh_outputs(), prec)))
        except Exception as e:  # reported below, on the main thread
            errors.append(e)

    threads = [threading.Thread(target=work, args=(i,)) for i in range(6)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    assert len(out) == 18
    for kind, r in out:
        if kind == "ne":
            for a, b in zip(r[0] + r[1], ne_ref[0] + ne_ref[1]):
                assert np.array_equal(a, b)
        else:
            for k in ("rad", "tau", "tp"):
                assert np.array_equal(getattr(r, k), getattr(ref[kind], k), equal_nan=True), (kind, k)
