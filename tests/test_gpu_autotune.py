"""cfd3d_autotune picks launch shapes by timing; the iterations it leaves behind give the
same states bit for bit as the default shapes (each thread's arithmetic is unchanged)."""
import numpy as np
import pytest

from cfd3d_gb300 import abi, cases, native

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [abi.FP64, abi.MIXED])
def test_autotune_choices_and_unchanged_results(precision):
    c = cases.make("batched", scale=8)
    c["cfg"]["fix_cav_clamp"] = 1
    out = []
    for tune in (False, True):
        e = native.Engine(c, precision=precision)
        e.initialize(c["pv0"])
        e.iterate(1, 1, 0.0)
        if tune:
            face, rhs, per_sm = e.autotune(2)
            assert face in (64, 128, 256) and rhs in (64, 128, 256) and per_sm >= 1
        for it in range(2):
            e.iterate(1, it + 2, 0.0)
        out.append([e.download(n)["pv"] for n in range(len(c["blocks"]))])
        e.close()
    for a, b in zip(*out):
        assert np.array_equal(a, b)
