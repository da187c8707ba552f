"""The correctly rounded library functions of crmath.cuh, built for the host:
every input's result equals the float64 evaluation rounded once to float32
(inputs too close to a rounding midpoint for float64 to decide are left out;
there are none or almost none)."""
import numpy as np
import pytest

import crcheck


@pytest.fixture(scope="module")
def host_cr(tmp_path_factory):
    return crcheck.host_library(str(tmp_path_factory.mktemp("cr")))


@pytest.mark.parametrize("fn", range(6), ids=crcheck.NAMES)
def test_host_build_is_correctly_rounded(host_cr, fn):
    x = crcheck.inputs(fn, 400_000)
    want, amb = crcheck.reference(fn, x)
    got = host_cr(fn, x)
    assert amb.sum() <= (0 if fn in (crcheck.POW5, crcheck.POW_M2) else 2)
    bad = (got != want) & ~amb
    assert not bad.any(), (x[bad][:5], got[bad][:5], want[bad][:5])


def test_inputs_cover_the_reduction_edges():
    x = crcheck.inputs(crcheck.SIN, 1000)
    # arguments within a few thousand ulps of multiples of pi/2 are present
    k = np.rint(x / np.float32(np.pi / 2))
    near = np.abs(x.astype(np.float64) - k * (np.pi / 2)) < 1e-3
    assert near.sum() > 100
