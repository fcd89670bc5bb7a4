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


def test_face_residual_pipeline_unchanged_results():
    """the mixed form's face stage and residual pipelined over 2, 4 and all blocks (the
    residual of one group on a second stream beside the face stage of the next) leave the
    same states, sweeps and norms bit for bit as the sequential stage"""
    c = cases.make("batched", scale=8)
    c["cfg"]["fix_cav_clamp"] = 1
    nb = len(c["blocks"])
    out = []
    for groups in (1, 2, 4, min(nb, 16)):
        e = native.Engine(c, precision=abi.MIXED)
        e.initialize(c["pv0"])
        shapes = list(e.launch_shapes())
        shapes[3] = groups
        e.set_launch_shapes(shapes)
        assert e.launch_shapes()[3] == groups
        norms = []
        for it in range(3):
            _, res, _ = e.iterate(1, it + 1, 0.0)
            norms.append(res)
        st = [e.download(n) for n in range(nb)]
        r0 = e.residual(0)["res"]
        out.append((norms, st, r0))
        e.close()
    base = out[0]
    for norms, st, r0 in out[1:]:
        assert np.array_equal(np.array(norms), np.array(base[0]))
        for a, b in zip(st, base[1]):
            for key in ("pv", "dv", "tv"):
                assert np.array_equal(a[key], b[key]), key
        assert np.array_equal(r0, base[2])


def test_set_launch_shapes_rejects_bad_values():
    c = cases.make("batched", scale=8)
    c["cfg"]["fix_cav_clamp"] = 1
    e = native.Engine(c, precision=abi.MIXED)
    good = list(e.launch_shapes())
    nb = len(c["blocks"])
    for bad in ([96, good[1], good[2], 1], [good[0], 512, good[2], 1], [good[0], good[1], 0, 1],
                [good[0], good[1], good[2], 0], [good[0], good[1], good[2], min(nb, 16) + 1]):
        with pytest.raises(RuntimeError):
            e.set_launch_shapes(bad)
        assert list(e.launch_shapes()) == good
    e.close()
    e64 = native.Engine(c, precision=abi.FP64)
    s64 = list(e64.launch_shapes())
    assert s64[3] == 1
    with pytest.raises(RuntimeError):
        e64.set_launch_shapes(s64[:3] + [2])
    e64.close()
