"""Host-side logic that needs no GPU: the bench's cross-rank reduction on two
gloo ranks, and the rta plugin built against the reference headers."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REFERENCE = os.environ.get("RTA_REFERENCE") or os.path.join(
    os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))), "reference")


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = bench.max_over_ranks(10.0 + 5.0 * rank, dist, "cpu")
    q.put((rank, t))
    dist.barrier()
    dist.destroy_process_group()


def test_bench_takes_the_max_over_two_gloo_ranks():
    import multiprocessing as mp
    import socket
    ctx = mp.get_context("spawn")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=5) for _ in range(2))
    assert got == [(0, 15.0), (1, 15.0)]


def test_single_process_max_is_identity():
    import bench
    assert bench.max_over_ranks(3.5) == 3.5


@pytest.mark.skipif(not os.path.isdir(REFERENCE) or shutil.which("g++") is None,
                    reason="reference headers not present")
def test_plugin_builds_and_exports_the_plugin_abi():
    """bbvh-gb300.so exports the four symbols rta's loader binds
    (librta/plugins.cpp:82-85)."""
    lib_so = os.path.join(ROOT, "rta_gb300", "_build", "librta_gb300.so")
    if not os.path.exists(lib_so):
        from rta_gb300 import build as B
        B.build()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "plugin"), f"REF={REFERENCE}"], check=True)
    so = os.path.join(ROOT, "plugin", "_build", "bbvh-gb300.so")
    out = subprocess.run(["nm", "-D", "--defined-only", so], capture_output=True, text=True,
                         check=True).stdout
    syms = {line.split()[-1] for line in out.splitlines() if line.strip()}
    assert {"description", "initialize", "parse_cmdline", "create_rt_set"} <= syms
