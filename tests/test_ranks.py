"""The multi-rank bookkeeping of bench.py (replicas, one per GPU) on CPU ranks: the
timed region's max over ranks by an all-reduce and the whole-job throughput, with
world_size 2 over gloo on 127.0.0.1."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = bench.max_over_ranks(1.0 + rank, "cpu")   # rank 1 is the slower one
    q.put((rank, t, bench.replica_throughput(world, 20, t)))
    dist.destroy_process_group()


def test_max_over_ranks_and_throughput_with_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [t for _, t, _ in out] == [2.0, 2.0]
    assert all(abs(v - 2 * 20 / 2.0) < 1e-12 for _, _, v in out)


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.replica_throughput(1, 20, 2.0) == 10.0


def test_reference_arm_prints_the_contract_line():
    """``bench.py --impl reference`` (the reference's own compiled formPT on the host
    cores; no GPU) prints one JSON line with the GPU arm's metric, unit and config and
    an e2e object without host-device traffic."""
    import json
    import subprocess
    if not os.path.isdir(os.path.join(ROOT, "oracle", "_ref", "mmd")):
        pytest.skip("the reference's compiled Cython (oracle/_ref) is not built here")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "1"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    if "unavailable" in line:
        return
    import bench
    assert line["metric"] == bench.METRIC and line["unit"] == "Fock builds/s"
    assert line["value"] > 0 and line["higher_is_better"] is True
    assert line["config"]["workload"] == bench.WORKLOAD["workload"]
    assert line["cpu_baseline"]["kind"] == "reference" and line["cpu_baseline"]["cores"] >= 1
    assert line["cpu_baseline"]["t_build_1core_s"] > 0 and line["cpu_baseline"]["quartets_per_s_1core"] > 0
    assert line["e2e"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
