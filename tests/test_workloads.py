"""CPU checks of the package's synthetic-data generators.

* The 1D initial fields and mesh (workloads.init_1d / mesh_1d, used by the
  shock and heat-transfer benchmarks) equal the oracle's restatement of
  initializer.c:296-424 and mesh_setup.c for every Init_field case.
* The Rankine-Hugoniot state of the shock family satisfies the jump
  conditions.
"""
import math

import numpy as np
import pytest

from spectralbte_gb300 import workloads as wl


@pytest.mark.parametrize("ic", [0, 1, 2, 3, 5, 6])
@pytest.mark.parametrize("order", [1, 2])
def test_init_1d_matches_oracle(oracle, ic, order):
    r = oracle.Run1D(8, 6.0, 10, order, ic, 1e-3, 1.0)
    a, b = r.init(), wl.init_1d(r.g.v, 10, order, ic)
    assert np.abs(a - b).max() <= 1e-15 * np.abs(a).max()
    x, dx = wl.mesh_1d(10, order)
    assert np.abs(x - r.x).max() < 1e-15 and np.array_equal(dx, r.dx)


def test_rankine_hugoniot_jump_conditions():
    from spectralbte_gb300.learned import rankine_hugoniot
    g = 5.0 / 3.0
    (r1, u1, t1), (r2, u2, t2) = rankine_hugoniot(1.2)
    assert math.isclose(u1, 1.2 * math.sqrt(5.0 / 3.0))
    assert math.isclose(r1 * u1, r2 * u2)                              # mass
    assert math.isclose(r1 * u1 * u1 + r1 * t1, r2 * u2 * u2 + r2 * t2)  # momentum
    e1 = 0.5 * u1 * u1 + g / (g - 1) * t1                              # enthalpy
    e2 = 0.5 * u2 * u2 + g / (g - 1) * t2
    assert math.isclose(e1, e2)
