"""cfd3d_upload_state / cfd3d_download_state (the t_variable accessors getpv/setpv..,
src/variable_module.f90:22-39): a seeded state goes in and comes back bit for bit, from
pinned and from pageable host memory, array by array, without touching the other block."""
import numpy as np
import pytest
import torch

from cfd3d_gb300 import abi, cases, native

pytestmark = pytest.mark.gpu


def _case():
    c = cases.split_i(cases.make("large", scale=16), 2)     # SST, cavitation, BDF2: nqq = 2
    return c


def _random_state(e, b, rng):
    blk = e.case["blocks"][b]
    return dict(pv=rng.normal(size=abi.padded_shape(blk, e.npv)),
                dv=rng.normal(size=abi.padded_shape(blk, 18)),
                tv=rng.normal(size=abi.padded_shape(blk, e.ntv)),
                qq=rng.normal(size=abi.interior_shape(blk, 2 * e.npv)))


def _pinned(a):
    t = torch.empty(a.size, dtype=torch.float64, pin_memory=True)
    v = t.numpy().reshape(a.shape)
    v[...] = a
    return t, v


@pytest.mark.parametrize("memory", ["pinned", "pageable"])
def test_round_trip_is_bit_exact(memory):
    c = _case()
    e = native.Engine(c)
    e.initialize(c["pv0"])
    assert e.nqq and e.ntv == 3 and len(c["blocks"]) == 2
    rng = np.random.default_rng(21)
    before = e.download(0)
    st = _random_state(e, 1, rng)
    keep = {k: _pinned(v) for k, v in st.items()} if memory == "pinned" else None
    src = {k: keep[k][1] for k in st} if keep else st
    e.upload(1, **src)
    got = e.download(1)
    for k in ("pv", "dv", "tv", "qq"):
        assert np.array_equal(got[k], st[k]), k
    # the other block is untouched
    after = e.download(0)
    for k in ("pv", "dv", "tv", "qq"):
        assert np.array_equal(after[k], before[k]), k
    # download into caller-owned pinned arrays, every field in one call
    out = {k: _pinned(np.zeros_like(v)) for k, v in st.items()}
    rcav = np.zeros(abi.interior_shape(c["blocks"][1], 2))
    e.download_arrays(1, pv=out["pv"][1], dv=out["dv"][1], tv=out["tv"][1], qq=out["qq"][1], rcav=rcav)
    for k in ("pv", "dv", "tv", "qq"):
        assert np.array_equal(out[k][1], st[k]), k
    assert np.array_equal(rcav, got["rcav"])


def test_partial_upload_leaves_the_rest():
    c = _case()
    e = native.Engine(c)
    e.initialize(c["pv0"])
    rng = np.random.default_rng(22)
    before = e.download(0)
    st = _random_state(e, 0, rng)
    e.upload(0, dv=st["dv"])
    got = e.download(0)
    assert np.array_equal(got["dv"], st["dv"])
    for k in ("pv", "tv", "qq"):
        assert np.array_equal(got[k], before[k]), k
    e.upload(0, tv=st["tv"], qq=st["qq"])
    got = e.download(0)
    assert np.array_equal(got["tv"], st["tv"]) and np.array_equal(got["qq"], st["qq"])
    assert np.array_equal(got["pv"], before["pv"])


@pytest.mark.parametrize("precision", [abi.FP64, abi.MIXED])
def test_upload_primitives_reproduces_the_iterated_state(precision):
    """cfd3d_upload_primitives: pv and qq of an iterated state set on a second engine give
    the interior dv and tv of the first bit for bit (the update's EOS and eddy viscosity),
    and the next iteration of both engines gives the same state"""
    c = _case()
    c["cfg"]["fix_cav_clamp"] = 1
    e1 = native.Engine(c, precision=precision)
    e1.initialize(c["pv0"])
    for it in range(2):
        e1.iterate(1, it + 1, 0.0)
    e2 = native.Engine(c, precision=precision)
    e2.initialize(c["pv0"])
    for b in range(2):
        s1 = e1.download(b)
        e2.upload_primitives(b, s1["pv"], s1["qq"])
        s2 = e2.download(b)
        core = (slice(3, -3), slice(3, -3), slice(3, -3))
        for k in ("dv", "tv"):
            assert np.array_equal(s2[k][core], s1[k][core]), k
        assert np.array_equal(s2["pv"], s1["pv"]) and np.array_equal(s2["qq"], s1["qq"])
    e1.iterate(1, 3, 0.0)
    e2.iterate(1, 3, 0.0)
    for b in range(2):
        s1, s2 = e1.download(b), e2.download(b)
        for k in ("pv", "dv", "tv"):
            assert np.array_equal(s2[k][3:-3, 3:-3, 3:-3], s1[k][3:-3, 3:-3, 3:-3]), (b, k)


def test_whole_case_transfers_equal_the_per_block_calls():
    """cfd3d_upload_primitives_all / cfd3d_download_state_all over every block give what
    the per-block calls give, bit for bit"""
    c = _case()
    c["cfg"]["fix_cav_clamp"] = 1
    e1 = native.Engine(c, precision=abi.MIXED)
    e1.initialize(c["pv0"])
    for it in range(2):
        e1.iterate(1, it + 1, 0.0)
    st = [e1.download(b) for b in range(2)]
    ea = native.Engine(c, precision=abi.MIXED)
    eb = native.Engine(c, precision=abi.MIXED)
    for e in (ea, eb):
        e.initialize(c["pv0"])
    ea.upload_primitives_all([np.ascontiguousarray(s["pv"]) for s in st], [np.ascontiguousarray(s["qq"]) for s in st])
    for b in range(2):
        eb.upload_primitives(b, st[b]["pv"], st[b]["qq"])
    for e in (ea, eb):
        e.iterate(1, 3, 0.0)
    outs = [dict(pv=np.zeros_like(s["pv"]), dv=np.zeros_like(s["dv"]), tv=np.zeros_like(s["tv"])) for s in st]
    ea.download_state_all([o["pv"] for o in outs], [o["dv"] for o in outs], [o["tv"] for o in outs])
    for b in range(2):
        ref = eb.download(b)
        for k in ("pv", "dv", "tv"):
            assert np.array_equal(outs[b][k], ref[k]), (b, k)


def test_whole_case_upload_takes_only_changed_cells():
    """cfd3d_upload_primitives_all of the engine's own state changes nothing (the cells whose
    pv is unchanged keep their dv and tv, which are the EOS of that pv); a cell whose pv the
    host changed gets the update's EOS, as the per-block call gives it; the next iteration
    matches an engine that took the same state through the per-block calls"""
    c = _case()
    c["cfg"]["fix_cav_clamp"] = 1
    e1 = native.Engine(c, precision=abi.MIXED)
    e1.initialize(c["pv0"])
    for it in range(2):
        e1.iterate(1, it + 1, 0.0)
    st = [e1.download(b) for b in range(2)]
    e1.upload_primitives_all([np.ascontiguousarray(s["pv"]) for s in st], [np.ascontiguousarray(s["qq"]) for s in st])
    for b in range(2):
        after = e1.download(b)
        for k in ("pv", "dv", "tv", "qq"):
            assert np.array_equal(after[k], st[b][k]), (b, k)
    # one interior cell of block 1 changed on the host
    pv = [np.ascontiguousarray(s["pv"]).copy() for s in st]
    pv[1][5, 5, 5, 0] += 250.0
    pv[1][5, 5, 5, 4] += 0.01
    e1.upload_primitives_all(pv, [np.ascontiguousarray(s["qq"]) for s in st])
    e2 = native.Engine(c, precision=abi.MIXED)
    e2.initialize(c["pv0"])
    for b in range(2):
        e2.upload_primitives(b, pv[b], st[b]["qq"])
    for b in range(2):
        a, r = e1.download(b), e2.download(b)
        for k in ("pv", "dv", "tv"):
            assert np.array_equal(a[k][3:-3, 3:-3, 3:-3], r[k][3:-3, 3:-3, 3:-3]), (b, k)
    e1.iterate(1, 3, 0.0)
    e2.iterate(1, 3, 0.0)
    for b in range(2):
        a, r = e1.download(b), e2.download(b)
        for k in ("pv", "dv", "tv"):
            assert np.array_equal(a[k][3:-3, 3:-3, 3:-3], r[k][3:-3, 3:-3, 3:-3]), (b, k)
