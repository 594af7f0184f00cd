"""bench.py's JSON contract on the CPU: the reference arm (the oracle port) on the small waveguide
workload, once as one process and once as two gloo ranks under torch.distributed.run (rank 0 prints
the only line), and the max-over-ranks reduction the timed regions use."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _json_lines(text):
    return [json.loads(l) for l in text.splitlines() if l.startswith("{")]


def _check_reference_line(d, n_gpus):
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["n_gpus"] == n_gpus and d["higher_is_better"] is True
    assert d["value"] > 0 and d["config"]["workload"] == "waveguide_small"
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1


def test_reference_arm_one_process():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "waveguide", "--steps", "1",
                        "--warmup", "0"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1
    _check_reference_line(lines[0], 1)


def test_reference_arm_two_gloo_ranks():
    pytest.importorskip("torch")
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py", "--impl",
                        "reference", "--workload", "waveguide", "--steps", "1", "--warmup", "0", "--gpus", "2"],
                       cwd=ROOT, capture_output=True, text=True, timeout=900, env=env)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1
    _check_reference_line(lines[0], 2)


def _max_worker(rank, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2")
    dist.init_process_group("gloo", rank=rank, world_size=2)
    sys.path.insert(0, ROOT)
    import bench

    v = bench.barrier_max(1.5 + rank, 2)
    bench.barrier(2)
    q.put((rank, v))
    dist.destroy_process_group()


def test_barrier_max_over_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_max_worker, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=300) for _ in range(2))
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert got == [(0, 2.5), (1, 2.5)]


def test_reference_arm_loads_no_product_library():
    """The reference arm builds its workload on the oracle's mesh and times only oracle code: the
    product's shared library must never be mapped into its process."""
    code = ("import sys, json; sys.argv=['bench.py','--impl','reference','--workload','waveguide','--steps','1',"
            "'--warmup','0']; import bench; bench.main(); maps=open('/proc/self/maps').read(); "
            "print('LOADED' if 'libfem2d_gb300' in maps else 'CLEAN')")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip().splitlines()[-1] == "CLEAN"
    line = _json_lines(r.stdout)[0]
    assert line["config"]["basis"] == "HierPoly" and line["config"]["glq"] == [8, 8]


def test_reference_arm_unavailable_line_from_fixture():
    """At the full-form 1M workload the committed oracle fixture's single-step time rules out a timed
    run of W + K steps: the arm prints one reasoned `unavailable` line and exits 0."""
    if not os.path.exists(os.path.join(ROOT, "tests", "golden", "full_form_full_1m.json")):
        pytest.skip("full_1m oracle fixture not generated")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "20", "--warmup", "5"],
                       cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1 and lines[0]["impl"] == "reference"
    assert "unavailable" in lines[0] and lines[0]["config"]["ndofs"] == 1070625


def test_workload_scripts_identical_on_oracle_and_product_meshes():
    sys.path.insert(0, ROOT)
    from fem_2d_gb300 import configs
    from oracle import ref

    for make in (lambda r: configs.precision(replay=r), lambda r: configs.waveguide_small(replay=r),
                 lambda r: configs.full_scale(seed=0, nx=16, ny=8, rounds=3, fraction=0.44, replay=r),
                 lambda r: configs.learned_family(4, 8, 4, replay=r), lambda r: configs.batch_member(3, replay=r)):
        assert make(configs.NativeReplay).ops == make(ref.OracleReplay).ops
