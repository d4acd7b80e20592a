"""bench.py --gpus N > 1: independent replicas, one simulation per GPU.  The
ranks share no data; the host-side helpers (device selection, barrier, max of
the timed region over ranks) are exercised here with two gloo ranks on CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_replica_device_mapping():
    sys.path.insert(0, ROOT)
    import bench
    # unset: the rank's own index
    assert bench.replica_device(0, None) == "0" and bench.replica_device(3, None) == "3"
    assert bench.replica_device(1, "4,5,6") == "5"
    assert bench.replica_device(0, " 7 , 2") == "7"
    # a list without an entry for the rank must not fall back to a GPU outside it
    with pytest.raises(RuntimeError, match="no device"):
        bench.replica_device(2, "4,5")
    with pytest.raises(RuntimeError, match="no device"):
        bench.replica_device(3, "4,5")
    # set but empty: every GPU is hidden, so no rank may pick one
    with pytest.raises(RuntimeError, match="no device"):
        bench.replica_device(0, "")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", RANK=str(rank),
                      LOCAL_RANK=str(rank), CUDA_VISIBLE_DEVICES="3,1")
    sys.path.insert(0, ROOT)
    import bench
    bench.replica_setup()
    assert os.environ["CUDA_VISIBLE_DEVICES"] == ("3", "1")[rank]
    bench.replica_barrier()
    m = bench.replica_max(10.0 + rank)
    out.put((rank, m, bench.world()))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_max():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 11.0, (2, 0)), (1, 11.0, (2, 1))]


def test_bench_reads_the_committed_traffic_captures():
    """roofline.traffic comes from the committed ncu summaries: both passes'
    per-launch DRAM bytes at 2048^2 and 4096^2, with the capture's build."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    for n in (2048, 4096):
        bench.apply_preset(1, "fp32", n)
        for key in ("row", "col"):
            traffic, src = bench.ncu_traffic(key)
            assert traffic and traffic > 1e6, (n, key)
            assert src.startswith(f"profiles/ncu_traffic_{n}x{n}_fp32.txt (build ")
