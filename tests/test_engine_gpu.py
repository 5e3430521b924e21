"""Retrieval engine (continuous batching, jgb_engine_*) on the GPU.

* A request's results are bit-identical whether it runs alone or admitted
  into a running mix of other requests of different sizes (levels, rays,
  channels), in FP64 and in mixed precision: every kernel of the engine
  works per request, forward models leave requests that are not part of a
  sub-step untouched, and the working-set rebuilds move state by copies.
* Admission respects the slot limit and the memory budget.
* FP64 engine results equal the CPU oracle's retrieval (restatement of
  optimal_estimation, retrieval.c:448-749, pinned to the reference build)
  within 1e-6 relative, iterations identical.
"""
import copy

import numpy as np
import pytest

from jurassic_gb300 import native, synth
from jurassic_gb300.model import Ret

pytestmark = pytest.mark.gpu


def _setup(nd=10, nreq=6, seed=21):
    w = synth.config_nadir(1, nd=nd, nlev=31, ztop=60.0, emitters=("CO2", "H2O"),
                           numin=660.0, numax=1600.0)
    ctl = copy.deepcopy(w.ctl)
    ctl.rett_zmin, ctl.rett_zmax = 0.0, 40.0
    ctl.retq_zmin = np.array([-999.0, 0.0])
    ctl.retq_zmax = np.array([-999.0, 14.0])
    from oracle import oracle
    ora = oracle.Oracle(ctl, w.tables, w.filters)
    rng = np.random.default_rng(seed)
    nch = rng.integers(nd // 2, nd + 1, nreq)
    items = synth.retrieval_requests(ctl, lambda b: ora.formod_batch(b.fresh_outputs()), nreq,
                                     seed, nlev=(21, 31), nch=nch)
    ret = Ret(kernel_recomp=1, conv_itmax=5, conv_dmin=0.01, err_ana=1,
              err_noise=np.full(ctl.nd, 1e-4), err_formod=np.full(ctl.nd, 0.5),
              err_temp=2.0, err_temp_cz=3.0, err_temp_ch=500.0,
              err_q=np.array([0.0, 30.0]), err_q_cz=np.array([-999.0, 3.0]),
              err_q_ch=np.array([-999.0, 500.0]))
    return ctl, w, ret, items, ora


KEYS = ("x", "costs", "rad", "tau", "tp", "p", "cov", "avk", "err_total", "err_noise",
        "err_formod", "cont", "res")


def _same(a, b):
    for k in KEYS:
        assert np.array_equal(np.asarray(a[k]), np.asarray(b[k]), equal_nan=True), k
    assert a["iters"] == b["iters"] and a["status"] == b["status"] == 0


@pytest.mark.parametrize("precision", [native.FP64, native.MIXED])
def test_same_alone_and_in_mix(built_lib, built_oracle, precision):
    ctl, w, ret, items, ora = _setup()
    ctx = native.Context(ctl, w.tables, w.filters)
    probe = 2
    alone = ctx.engine(ret, precision).run(synth.pack(ctl, [items[probe]]))[0]
    # a running mix: two requests start, the probe joins one step later, the
    # others one step after that; at most 4 in flight
    eng = ctx.engine(ret, precision, max_active=4)
    first = eng.submit(synth.pack(ctl, items[:2]))
    eng.step()
    pid = eng.submit(synth.pack(ctl, [items[probe]]))[0]
    eng.step()
    eng.submit(synth.pack(ctl, items[3:]))
    out = {}
    for _ in range(200):
        eng.step()
        for rid in eng.finished():
            out[rid] = eng.result(rid)
        if len(out) == len(items):
            break
    assert pid in out and all(r in out for r in first)
    st = eng.stats()
    assert st["finished"] == len(items) and st["failed"] == 0
    assert st["rebuilds"] >= 3      # requests joined and left between steps
    _same(alone, out[pid])


def test_slot_limit_and_budget(built_lib, built_oracle):
    ctl, w, ret, items, ora = _setup(nreq=5)
    ctx = native.Context(ctl, w.tables, w.filters)
    ref = ctx.engine(ret, native.FP64).run(synth.pack(ctl, items))
    for kw, cap in ((dict(max_active=2), 2), (dict(mem_budget=1), 1)):
        eng = ctx.engine(ret, native.FP64, **kw)
        ids = eng.submit(synth.pack(ctl, items))
        got = {}
        while len(got) < len(ids):
            a, q, d = eng.step()
            assert a <= cap
            assert eng.stats()["active"] <= cap
            for rid in eng.finished():
                got[rid] = eng.result(rid)
        for i, rid in enumerate(ids):
            _same(ref[i], got[rid])


def test_engine_fp64_vs_oracle(built_lib, built_oracle):
    ctl, w, ret, items, ora = _setup(nreq=4)
    ctx = native.Context(ctl, w.tables, w.filters)
    res = ctx.engine(ret, native.FP64).run(synth.pack(ctl, items))
    for i, (a, o) in enumerate(items):
        r = ora.retrieval(ret, a, o)
        assert np.max(np.abs(res[i]["x"] - r["x"]) / np.maximum(np.abs(r["x"]), 1e-300)) <= 1e-6, i
        assert res[i]["iters"] == r["iters"], i
        assert np.allclose(res[i]["costs"], r["costs"], rtol=1e-6), i
        assert np.max(np.abs(res[i]["cov"] - r["cov"])) <= 1e-6 * np.max(np.abs(r["cov"])), i
        # standard deviation of the total error is the covariance diagonal
        assert np.allclose(res[i]["err_total"], np.sqrt(np.diag(res[i]["cov"])), rtol=1e-14)


def test_mixed_engine_within_posterior_sigma(built_lib, built_oracle):
    ctl, w, ret, items, ora = _setup(nreq=4)
    ctx = native.Context(ctl, w.tables, w.filters)
    r64 = ctx.engine(ret, native.FP64).run(synth.pack(ctl, items))
    r32 = ctx.engine(ret, native.MIXED).run(synth.pack(ctl, items))
    for a, b in zip(r64, r32):
        assert np.max(np.abs(a["x"] - b["x"]) / a["err_total"]) <= 0.05
