"""The CUDA library reproduces the golden fixtures through the C ABI: cell and
contact lists bit for bit; parcel, body and field values after two steps to
1e-9 relative (the body rotation uses CUDA's cos/sin)."""
import pytest

import golden_util

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", golden_util.NAMES)
def test_gpu_matches_golden(gpu_lib, name):
    d, inputs = golden_util.load(name)
    case = gpu_lib.Case(*inputs, device=0)
    golden_util.check(case, d, rtol_bodies=1e-9)
    case.close()
