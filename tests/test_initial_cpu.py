"""Initial states (specmc_gb300.initial) against the reference's
core/bench_ic.py and physics/heating.py (tests/golden/initial_32x24.npz,
written by the reference on the seeded synthetic ASPECT-layout file
tests/golden/aspect_synthetic.txt).  The functions need only a model's
x, z, coeffs and seed; the oracle's model, pinned to the reference's
transforms, provides them here."""
import os

import numpy as np
import pytest

from oracle import specmc_oracle as O

from conftest import GOLDEN


def _rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


@pytest.fixture(scope="module")
def ref():
    return np.load(os.path.join(GOLDEN, "initial_32x24.npz"))


def test_initial_states_match_reference(ref):
    from specmc_gb300 import initial as I
    m = O.ConstModel(Ra=1e4, Nx=32, Nz=24)
    path = os.path.join(GOLDEN, "aspect_synthetic.txt")
    assert _rel(I.conductive_theta(m, amp=3e-2, m=2, n=1), ref["conductive"]) < 1e-14
    assert _rel(I.analytic_bl_theta(m), ref["analytic_bl"]) < 1e-13
    assert _rel(I.heated_conductive_theta(m.z, 1.5), ref["heated"]) < 1e-15
    assert _rel(I.aspect_theta(m, path=path), ref["aspect_pchip"]) < 1e-12
    assert _rel(I.aspect_theta(m, path=path, zinterp="spline"), ref["aspect_spline"]) < 1e-12
    assert _rel(I.ic_theta(m, "aspect", path=path), ref["aspect_pchip"]) < 1e-12
    assert _rel(I.ic_theta(m, "bl"), ref["analytic_bl"]) < 1e-13


def test_initial_state_errors(tmp_path):
    from specmc_gb300 import initial as I
    m = O.ConstModel(Ra=1e4, Nx=32, Nz=24)
    with pytest.raises(FileNotFoundError):
        I.find_aspect_ic(str(tmp_path / "missing.txt"))
    bad = tmp_path / "bad.txt"
    bad.write_text("# POINTS: 4 4\n0 0 1\n")
    with pytest.raises(ValueError):
        I.read_aspect_ic(str(bad))
    with pytest.raises(ValueError):
        I.aspect_theta(m, path=os.path.join(GOLDEN, "aspect_synthetic.txt"), zinterp="poly")
    with pytest.raises(ValueError):
        I.ic_theta(m, "nope")
