"""The oracle against the committed regression fixtures (no GPU).

tests/golden/*.npz hold the oracle's own outputs on small seeded cases
(tests/golden/make_golden.py): one V-cycle and one time step of CH 2D
periodic, CH 3D Dirichlet, BioGrowth 2D and the three-variable growth
plugin, and F25.12 text.  The reference has no tests to take fixtures from;
these pin the oracle against changes of itself, bit for bit.
"""
import os

import numpy as np
import pytest

from tests.golden import make_golden as mg

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("name", sorted(mg.CASES))
def test_oracle_reproduces_its_fixture(name):
    z = np.load(os.path.join(HERE, name + ".npz"))
    qv, qs, res, ncyc = mg.run(name, {"q": z["q"], "qold": z["qold"], "f": z["f"]})
    assert np.array_equal(qv, z["q_vcycle"])
    assert np.array_equal(qs, z["q_step"])
    assert ncyc == int(z["ncycles"]) and np.array_equal(res, z["residuals"])


def test_f25_fixture(oracle_mod, pkg):
    z = np.load(os.path.join(HERE, "f25.npz"))
    for v, t in zip(z["values"], z["text"]):
        assert oracle_mod.format_f25(float(v)) == str(t)
        assert pkg.format_f25(float(v)) == str(t)
