"""The CUDA library (through the C ABI) against the reference's own subroutines: the
plain FP64 method must reproduce the fixtures of tests/golden/ bit for bit, through the
eight stage kernels and through the fused step."""
import numpy as np
import pytest

import golden_cases as gc
from lbmgpu import Lattice

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", ["fused", "stages"])
@pytest.mark.parametrize("name", sorted(gc.cases()))
def test_library_reproduces_reference_steps(name, mode):
    meta = gc.cases()[name]
    p = gc.params_for(meta)
    data = gc.load(name)
    g = Lattice(p)
    g.initial()
    for f in gc.field_names(data):
        g.set_state(f, data["in_" + f])
    if mode == "fused":
        g.step(meta["steps"])
    else:
        for _ in range(meta["steps"]):
            g.stage_step()
    for f in gc.field_names(data):
        got = g.get_state(f)
        want = data["out_" + f]
        assert np.array_equal(got, want), (name, f, float(np.abs(got - want).max()))
