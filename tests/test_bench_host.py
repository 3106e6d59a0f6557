"""Host-side pieces of bench.py: the replica barrier / max-over-ranks helper
under a 2-rank gloo group, and the reference arm on a small airbox."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist(world)
    d.barrier()
    q.put((rank, d.max(float(rank + 1)), d.sum(float(rank + 1))))
    d.close()


def test_dist_helper_two_ranks_gloo():
    pytest.importorskip("torch")
    import multiprocessing as mp
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
    assert out == [(0, 2.0, 3.0), (1, 2.0, 3.0)]


def test_reference_arm_prints_one_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "config1",
                        "--steps", "1", "--warmup", "0"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "MLUPS" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0


def test_network_flop_count_matches_the_layer_list():
    """bench.net_flops (the multiply-adds behind --study net's TFLOP/s) against the network's layer list in the
    restatement: forward, data gradient (not for the first layer) and weight gradient of every convolution."""
    sys.path.insert(0, ROOT)
    import bench
    from oracle import warmstart_ref as R_
    for res, base, levels, batch in ((64, 16, 4, 8), (32, 8, 2, 2), (16, 8, 3, 1)):
        out_res = []
        for l in range(levels):
            out_res += [res >> l] * 2
        for l in range(levels - 2, -1, -1):
            out_res += [res >> l] * 2
        out_res.append(res)
        layers = R_.conv_layers(base, levels)
        assert len(layers) == len(out_res)
        want = sum(2.0 * 27 * cin * cout * d ** 3 * batch * (2 if i == 0 else 3)
                   for i, ((cin, cout, s, relu), d) in enumerate(zip(layers, out_res)))
        assert bench.net_flops(res, base, levels, batch) == pytest.approx(want, rel=1e-12)


def test_fixed_budget_rules_run_exactly_their_budget():
    """--warm-rules budget: two windows of A/2 steps after S settling steps, a tolerance no window misses."""
    sys.path.insert(0, ROOT)
    import bench
    for r in bench.BUDGET_RULES:
        assert r["max_steps"] == r["settle"] + 2 * r["window"] == r["settle"] + r["min_avg"]
        assert r["rule"] == 0 and r["tol"] > 1e6
    assert [r["settle"] + r["min_avg"] for r in bench.BUDGET_RULES] == [1250, 1500, 2000, 3000]
