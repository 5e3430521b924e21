"""Lifetimes of contexts, engines and call scratch on the GPU.

* An engine may outlive its context: destroying the context frees the
  engine's device memory with its own, the engine's calls then fail with
  JGB_ERR_STATE, and destroying the engine afterwards is safe.
* Repeated jgb_kernel calls allocate nothing that outlives the call (the
  device's free memory is the same after the second and the third call).
* A context with everything allocated (forward model, Jacobians, an
  engine) gives all of its device memory back when it is destroyed.
"""
import copy
import ctypes as C

import numpy as np
import pytest

from jurassic_gb300 import native, synth
from jurassic_gb300.model import Ret

pytestmark = pytest.mark.gpu

SLACK = 2 << 20  # bytes: the allocator's granularity


def free_bytes():
    """cudaMemGetInfo of the current device, through the CUDA runtime the
    library itself is linked with."""
    rt = C.CDLL("libcudart.so.13")
    free, total = C.c_size_t(0), C.c_size_t(0)
    assert rt.cudaMemGetInfo(C.byref(free), C.byref(total)) == 0
    return free.value


def _setup():
    w = synth.config_nadir(2, nd=8, nlev=31, ztop=60.0, emitters=("CO2", "H2O"),
                           numin=660.0, numax=1600.0)
    ctl = copy.deepcopy(w.ctl)
    ctl.rett_zmin, ctl.rett_zmax = 0.0, 40.0
    ctl.retq_zmin = np.array([-999.0, 0.0])
    ctl.retq_zmax = np.array([-999.0, 14.0])
    ret = Ret(kernel_recomp=1, conv_itmax=3, conv_dmin=0.01, err_ana=1,
              err_noise=np.full(ctl.nd, 1e-4), err_formod=np.full(ctl.nd, 0.5),
              err_temp=2.0, err_temp_cz=3.0, err_temp_ch=500.0,
              err_q=np.array([0.0, 30.0]), err_q_cz=np.array([-999.0, 3.0]),
              err_q_ch=np.array([-999.0, 500.0]))
    return w, ctl, ret


def _requests(ctx, ctl, w):
    meas = ctx.formod_batch(w.batch.fresh_outputs(), native.FP64)
    b = w.batch.fresh_outputs()
    b.rad = meas.rad.copy()
    return b


def _use_everything(ctx, ctl, w, ret):
    b = _requests(ctx, ctl, w)
    ctx.formod_batch(w.batch.fresh_outputs(), native.MIXED)
    ctx.kernel_batch(b, native.MIXED)
    eng = ctx.engine(ret, native.MIXED)
    eng.submit(b)
    eng.step()
    return eng


def test_engine_outlives_context(built_lib):
    w, ctl, ret = _setup()
    ctx = native.Context(ctl, w.tables, w.filters)
    eng = _use_everything(ctx, ctl, w, ret)
    ctx.close()
    with pytest.raises(native.JurassicError):
        eng.step()
    with pytest.raises(native.JurassicError):
        eng.stats()
    eng.close()
    eng.close()


def test_kernel_calls_keep_nothing(built_lib):
    w, ctl, ret = _setup()
    ctx = native.Context(ctl, w.tables, w.filters)
    b = _requests(ctx, ctl, w)
    ctx.kernel_batch(b, native.MIXED)
    ctx.kernel_batch(b, native.MIXED)
    f2 = free_bytes()
    for _ in range(3):
        ctx.kernel_batch(b, native.MIXED)
    assert free_bytes() >= f2 - SLACK
    ctx.close()


@pytest.mark.parametrize("engine_first", [True, False])
def test_destroy_gives_memory_back(built_lib, engine_first):
    w, ctl, ret = _setup()
    # a first context loads the kernels (module memory stays with the process)
    ctx = native.Context(ctl, w.tables, w.filters)
    _use_everything(ctx, ctl, w, ret).close()
    ctx.close()
    f0 = free_bytes()
    ctx = native.Context(ctl, w.tables, w.filters)
    eng = _use_everything(ctx, ctl, w, ret)
    assert free_bytes() < f0 - SLACK  # it did allocate
    if engine_first:
        eng.close()
        ctx.close()
    else:
        ctx.close()
        eng.close()
    assert free_bytes() >= f0 - SLACK
