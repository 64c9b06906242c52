"""The GPU path against the reference's own outputs (tests/golden/ref_pins.npz,
made by tests/golden/make_ref_pins.py from NaiveFracturer::buildCPU compiled
from the reference): the naive fracturer (vf_fracture with VF_NAIVE) through
the C ABI, bit for bit."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_pins.npz")


@pytest.mark.parametrize("gi", [0, 1, 2])
@pytest.mark.parametrize("dfunc", [0, 1, 2])
def test_gpu_naive_matches_reference(vf, ctx, gi, dfunc):
    pins = np.load(GOLD)
    grid, seeds = pins[f"naive{gi}_grid"], pins[f"naive{gi}_seeds"]
    g = vf.RegularGrid(grid.shape, None, None, ctx)
    g.upload(grid)
    fr = vf.NaiveFracturer()
    fr.setDistanceFunction(dfunc)
    fr.build(g, seeds)
    assert np.array_equal(g.data(), pins[f"naive{gi}_labels{dfunc}"])
    g.close()
