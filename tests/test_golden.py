"""The CPU restatement reproduces the committed golden fixtures (regression
pin; tests/golden/make_golden.py regenerates them)."""
import pytest

import golden_util


@pytest.mark.parametrize("name", golden_util.NAMES)
def test_oracle_matches_golden(oracle_mod, name):
    d, inputs = golden_util.load(name)
    case = oracle_mod.OracleCase(*inputs)
    golden_util.check(case, d, rtol_bodies=1e-12)
