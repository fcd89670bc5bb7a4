"""Host-side logic that needs no GPU: the input.inp reader, the synthetic cases, the
benchmark's byte model and its replica reduction (gloo, two ranks)."""
import os
import subprocess
import sys

import numpy as np
import pytest

from cfd3d_gb300 import abi, cases
from cfd3d_gb300.config import read_input, write_input

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_input_roundtrip():
    cfg = cases.make("cavitating", scale=16)["cfg"]
    back, bad = read_input(write_input(cfg, name="cav"))
    assert bad == []
    assert back["name"] == "cav"
    for k, v in cfg.items():
        if k in back:
            assert back[k] == pytest.approx(v, rel=1e-15), k


def test_input_flags_unsupported_options():
    cfg = dict(cases.make("plain_small", scale=16)["cfg"])
    text = write_input(cfg).splitlines()
    # gravity / csf value line is the 20th line (10th label/value pair): both are engine options
    text[19] = "1 1"
    back, bad = read_input("\n".join(text) + "\n")
    assert bad == [] and back["gravity"] == 1 and back["csf"] == 1
    # iread / rstnum (2nd pair): a restart, which the solve loop takes, not the engine
    text[3] = "1 5"
    _, bad = read_input("\n".join(text) + "\n")
    assert bad == ["iread"]


def test_fortran_real_literals():
    cfg = dict(cases.make("plain_small", scale=16)["cfg"])
    text = write_input(cfg)
    assert "d" in text  # reals are written as Fortran double literals
    back, _ = read_input(text.replace("d", "D"))
    assert back["pref"] == pytest.approx(cfg["pref"])


@pytest.mark.parametrize("name,cells", [("plain_small", 64 * 32 * 32), ("cavitating", 128 * 64 * 64),
                                        ("adjoint", 64 ** 3), ("large", 384 * 192 * 192)])
def test_case_sizes(name, cells):
    # generated at 1/8 resolution; the full-size count follows from the divisor
    c = cases.make(name, scale=8)
    assert cases.total_cells(c) * 8 ** 3 == cells
    for b, pv in zip(c["blocks"], c["pv0"]):
        assert pv.shape == abi.interior_shape(b, abi.sizes(c["cfg"])[0])
        assert np.all(np.isfinite(pv))
        assert np.all((pv[..., 5] >= 0.0) & (pv[..., 5] <= 1.0))


def test_batched_connections_are_point_matched():
    c = cases.make("batched", scale=8, nblocks=12)
    blocks = c["blocks"]
    for n, b in enumerate(blocks):
        for con in b["con"]:
            d = blocks[con["donor"]]
            back = [cc for cc in d["con"] if cc["donor"] == n]
            assert len(back) == 1
            assert tuple(back[0]["pnts"]) == tuple(con["pnts_donor"])
            # the shared face has the same node coordinates on both sides
            i0 = con["pnts"][0] - 1
            j0 = con["pnts_donor"][0] - 1
            assert np.array_equal(b["xyz"][:, :, i0], d["xyz"][:, :, j0])


@pytest.mark.parametrize("name,bytes_", [("plain_small", 728), ("cavitating", 776), ("adjoint", 896),
                                         ("large", 1040)])
def test_algorithmic_bytes_per_cell_iteration(name, bytes_):
    assert bench.algorithmic_bytes(cases.make(name, scale=16)["cfg"]) == bytes_


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference"],
                       capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 0
    assert r.stdout.strip() == ""


def _replica_rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms, value = bench.combine_ranks(10.0 * (rank + 1), 1000, dist)
    out.put((rank, ms, value))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_reduction_two_ranks_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 2000)
    procs = [ctx.Process(target=_replica_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    # slowest rank's time, whole-job throughput = 2 replicas x 1000 cells / 20 ms
    for rank, ms, value in got:
        assert ms == 20.0
        assert value == pytest.approx(2 * 1000 / 20.0 / 1e3)


def test_split_i_decomposition():
    c = cases.make("large", scale=16)
    s = cases.split_i(c, 4)
    assert len(s["blocks"]) == 4
    assert cases.total_cells(s) == cases.total_cells(c)
    assert np.array_equal(np.concatenate(s["pv0"], axis=2), c["pv0"][0])
    # interface nodes are shared; far-field patches only on the outer i faces
    for q, b in enumerate(s["blocks"]):
        iface = [bc for bc in b["bc"] if bc[1][0] == bc[1][3]]
        assert len(iface) == (1 if q in (0, 3) else 0)
        assert len(b["con"]) == (1 if q in (0, 3) else 2)
    for a, b in zip(s["blocks"][:-1], s["blocks"][1:]):
        assert np.array_equal(a["xyz"][:, :, -1, :], b["xyz"][:, :, 0, :])


def test_reference_arm_runs_the_gpu_arms_workload():
    """--impl reference times the CPU oracle on the GPU arm's workload: the same case, cut
    into the same blocks (one per host thread)"""
    import json
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--scale", "16",
                        "--blocks", "4", "--steps", "1", "--warmup", "1", "--ref-threads", "4"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    c = bench.workload("large", 16, 4)
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["config"]["blocks"] == 4 and line["config"]["cells"] == cases.total_cells(c)
    assert line["config"]["workload"] == bench.describe(c, cases.total_cells(c))
    assert line["e2e"]["h2d_bytes_per_step"] == 0
