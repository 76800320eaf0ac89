"""The multi-rank side of bench.py on CPU.  With N GPUs the bench runs one rank per GPU,
each imaging its own batch (replicas, no data-path collective); the step time is the
slowest rank's and the job throughput counts every rank's images.  Two gloo ranks check
that reduction and formula; the reference arm's non-zero ranks leave without work."""
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, times, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = bench.max_over_ranks(dist, times[rank], "cpu")
        out.put((rank, t, bench.job_images_per_s(world, 64, 10, t)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    times = [0.75, 1.25]
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        res = sorted(q.get(timeout=180) for _ in range(2))
    finally:
        for p in procs:
            p.join(timeout=60)
    assert [p.exitcode for p in procs] == [0, 0]
    assert [r[1] for r in res] == [1.25, 1.25]
    for _, _, v in res:
        assert abs(v - 2 * 64 * 10 / 1.25) < 1e-9


def test_single_process_keeps_its_own_time():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(None, 3.5, "cpu") == 3.5
    assert bench.job_images_per_s(1, 64, 20, 0.5) == 64 * 20 / 0.5


def test_reference_arm_nonzero_rank_exits_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1"], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
