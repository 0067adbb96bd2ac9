"""The oracle against golden vectors of the reference's own CPU
bound-and-split (tests/golden/, written by tests/golden/make_golden.py from
the reference's src/base/Patch.cpp and Projection.cpp): the same sub-patches,
bit for bit, in the same emission order."""
import numpy as np
import pytest

from helpers import GOLDEN_CASES, golden_case


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_oracle_matches_golden(built, name):
    from oracle import oracle
    sc, opts, gpid, grng = golden_case(name)
    pid, rng, _ = oracle.bound_n_split(sc, 0, params=oracle.make_params(sc, **opts))
    assert len(gpid) > 0
    assert np.array_equal(pid, gpid)
    assert np.array_equal(rng.view(np.uint32), grng.view(np.uint32))
