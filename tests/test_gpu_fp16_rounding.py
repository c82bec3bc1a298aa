"""Rounding of FP16 population storage.

At the bench workload (128^3, Ra 1e7, seeded 1e-3 noise in T) a step moves the stored
FP16 deviations by ~1e-8 while their unit in the last place is ~1e-6: round-to-nearest
drops every such increment and the lattice stays conductive (Nu ~ 1 after 20,000 steps,
where FP32 storage and FP64 reach Nu ~ 50 in the transient).  Stochastic rounding, the FP16
default, keeps the increments in expectation and convection develops.  Its random bits are
keyed on (step counter, cell, direction): a run is reproducible, and a continuation restart
carries the counter (the restart tests cover FP16)."""
import numpy as np
import pytest

from lbmgpu import LBM_OPT_FP16_ROUNDING, Lattice, LbmError
from lbmgpu.abi import rb_params

pytestmark = pytest.mark.gpu


def nu_after(steps, rounding):
    p = rb_params(dim=3, n=128, Ra=1e7, precision="fp16", noise_amp=1e-3)
    lat = Lattice(p)
    if rounding is not None:
        lat.set_option(LBM_OPT_FP16_ROUNDING, rounding)
    lat.initial()
    lat.step(steps)
    nu, re = lat.calNuRe()
    lat.close()
    return nu, re


def test_stochastic_rounding_lets_convection_start():
    nu_sr, re_sr = nu_after(20000, None)     # default: stochastic
    nu_rn, re_rn = nu_after(20000, 0)
    assert nu_sr > 5.0 and re_sr > 100.0, (nu_sr, re_sr)
    assert nu_rn < 1.5 and re_rn < 20.0, (nu_rn, re_rn)


def test_stochastic_rounding_is_reproducible():
    p = rb_params(dim=3, n=24, Ra=1e6, precision="fp16", noise_amp=1e-3, seed=5)
    runs = []
    for _ in range(2):
        lat = Lattice(p)
        lat.initial()
        lat.step(77)
        runs.append(lat.get_state("f"))
        lat.close()
    assert np.array_equal(runs[0], runs[1])


def test_rounding_option_only_for_fp16():
    lat = Lattice(rb_params(dim=3, n=12, Ra=1e6, precision="fp32"))
    with pytest.raises(LbmError):
        lat.set_option(LBM_OPT_FP16_ROUNDING, 1)
