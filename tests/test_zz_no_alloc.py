"""cfd3d_eos_eval_noalloc: the pointwise EOS through the library's static device buffer
gives the same results as cfd3d_eos_eval on two calls in a row, and rejects inputs larger
than the buffer before any device work.  Collected last so that it also runs after every
other test has used the device."""
import numpy as np
import pytest

from cfd3d_gb300 import abi, native
from cfd3d_gb300.native import Cfd3dError

pytestmark = pytest.mark.gpu


def _points(seed, n):
    rng = np.random.default_rng(seed)
    p = rng.uniform(2e3, 3e5, n)
    t = rng.uniform(280.0, 320.0, n)
    y1 = rng.uniform(0.0, 0.5, n) * (rng.uniform(size=n) < 0.5)
    y2 = 10.0 ** rng.uniform(-7, -3, n)
    return p, t, y1, y2


@pytest.mark.parametrize("fluid,prop", [(2, True), (2, False), (1, True)])
def test_noalloc_matches_allocating_entry_point_twice(fluid, prop):
    for seed, n in ((11, native.EOS_NOALLOC_MAX), (12, 777)):
        pts = _points(seed, n)
        dv_a, tv_a = native.eos_eval(*pts, fluid=fluid, prop=prop)
        dv_b, tv_b = native.eos_eval_noalloc(*pts, fluid=fluid, prop=prop)
        assert np.array_equal(dv_a, dv_b)
        if prop:
            assert np.array_equal(tv_a, tv_b)


def test_noalloc_rejects_oversize_input():
    pts = _points(13, native.EOS_NOALLOC_MAX + 1)
    with pytest.raises(Cfd3dError) as ei:
        native.eos_eval_noalloc(*pts)
    assert ei.value.code == abi.ERR_ARG
    # the buffer is untouched by the rejected call and still serves the next one
    pts = _points(14, 5)
    dv_a, _ = native.eos_eval(*pts)
    dv_b, _ = native.eos_eval_noalloc(*pts)
    assert np.array_equal(dv_a, dv_b)
