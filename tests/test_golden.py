"""The oracle against its committed golden fixtures (tests/golden/make_golden.py)."""

from pathlib import Path

import numpy as np
import pytest

from oracle import oracle
from tests.golden import make_golden

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("name", sorted(make_golden.CASES))
def test_oracle_reproduces_golden(name):
  ref = np.load(GOLDEN / f"{name}.npz")
  out = make_golden.render(name)
  np.testing.assert_array_equal(out["seg"], ref["seg"])
  np.testing.assert_array_equal(out["depth"], ref["depth"])
  diff = np.abs(oracle.unpack_rgb(out["rgb"]) - oracle.unpack_rgb(ref["rgb"]))
  assert diff.max() <= 1
  np.testing.assert_allclose(out["hdr"], ref["hdr"], rtol=1e-4, atol=1e-4 * float(np.abs(ref["hdr"]).max()))
