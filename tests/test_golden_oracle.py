"""The oracle reproduces the reference's own outputs stored in tests/golden/.

The fixtures were produced by the reference's C sources compiled unchanged
(tests/golden/make_golden.py); they carry the exact mesh tables the reference
saw, so this pins the oracle on any host, including ones without the
reference tree.  Comparison is bit for bit.
"""
import pytest

from fvtest import bits_equal, golden_names, load_golden
from pyoracle import Oracle


@pytest.mark.parametrize("name", golden_names())
def test_oracle_matches_reference_golden(name):
    t, cfg, z = load_golden(name)
    orc = Oracle(t, cfg)
    U = z["U"]
    if cfg.ischeme == 2:
        assert bits_equal(orc.faceinterp(U), z["SF"])
    if cfg.ns == 1:
        assert bits_equal(orc.gradcalc(U), z["SG"])
    assert bits_equal(orc.residual(U), z["R"])
    S = orc.step(U, float(z["dt"]), str(z["scheme"]), int(z["nsteps"]))
    assert bits_equal(S, z["S_out"])
    assert orc.error()[0] == 0
