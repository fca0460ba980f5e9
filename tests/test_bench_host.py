"""Host side of bench.py without a GPU: the reference arm's JSON line (the
reference's CG restated by the oracle, on the host cores) on a small grid,
the clock / throttle-reason parser of the sampled nvidia-smi log, and the
U-Net FLOP count behind the tensor roofline."""
import json
import subprocess
import sys

import pytest

from conftest import ROOT

sys.path.insert(0, str(ROOT))
import bench  # noqa: E402


def test_reference_arm_line(built):
    out = subprocess.run(
        [sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--size", "32",
         "--steps", "1", "--warmup", "0"],
        cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
                "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC and line["unit"] == bench.UNIT
    assert line["higher_is_better"] is False
    assert line["value"] > 0 and line["steps"] == 1 and line["warmup"] == 0
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    assert line["config"]["grid"] == [32, 32, 32]
    # the iteration count each bounded step is scaled to comes from a full
    # oracle solve of the same problem in the same run
    fs = line["full_solve"]
    assert fs["iterations"] > 0 and fs["s"] > 0 and fs["final_rel_res"] <= 1e-8
    assert f"{fs['iterations']} iterations of a full oracle solve" in cb["sample"]


def test_oracle_thread_count_is_settable_and_restored(built):
    from oracle import sbm_oracle as orc
    lib = orc.lib()
    n0 = lib.orc_num_threads()
    assert bench._orc_threads(1) == 1
    assert bench._orc_threads(0) == n0


def test_oracle_rate_scales_a_sample_to_the_measured_count(built):
    from elsim_gb300 import synth
    from oracle import sbm_oracle as orc
    m = synth.microstructure((24, 24, 24), seed=3, reinit_steps=20, redist=orc.redist)
    prob = synth.potential_problem(m["psi"])
    t_full, x, info = bench.oracle_solve(prob)
    assert info["status"] == 0 and info["iters"] > 10
    est, s = bench.oracle_rate(prob, 1e-9, info["iters"], threads=1)
    # the smallest sample (3 iterations), scaled to the full count
    assert s["iters"] == 3 and s["full_iters"] == info["iters"] and s["threads"] == 1
    assert est == pytest.approx(s["seconds"] / 3 * info["iters"])


class _Done:
    """Stands in for the nvidia-smi process the sampler stops."""

    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0

    def kill(self):
        pass


def _clocks(lines):
    c = bench.Clocks()
    c.f.write("".join(ln + "\n" for ln in lines))
    c.f.flush()
    c.p = _Done()
    return c.stop()


def test_clock_parser_median_and_reasons():
    ok = "0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active"
    capped = "0, 1980, 2070, 1390.5, 0x4, Not Active, Not Active, Not Active, Active"
    slow = "0, 1500, 2070, 700.0, 0x8, Active, Not Active, Not Active, Not Active"
    r = _clocks([ok, ok, capped])
    assert r["sm_mhz"] == 2070.0 and r["sm_max_mhz"] == 2070.0 and r["samples"] == 3
    assert r["reasons"] == ["sw_power_cap"]
    r = _clocks([ok, slow, "garbage line", "0, n/a, 2070"])
    assert r["samples"] == 2 and r["reasons"] == ["hw_slowdown"]
    assert r["sm_mhz"] == pytest.approx((2070.0 + 1500.0) / 2)


def test_clock_parser_without_samples():
    r = _clocks([])
    assert r["sm_mhz"] is None and r["samples"] == 0 and r["reasons"] == []


def test_unet_flops():
    # 2 * cin * cout * 27 * voxels over the nine 3x3x3 layers at 64^3 coarse
    want = sum(2 * ci * co * 27 * (64 >> lev) ** 3 for ci, co, lev in bench.UNET)
    assert bench.unet_flops(256) == want == 20_019_806_208
    assert bench.unet_flops(128) * 8 == bench.unet_flops(256)


def _max_worker(rank, port, q):
    import torch
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    import bench as b

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=2)
    try:
        q.put((rank, b._max_over_ranks(1.5 + 2.0 * rank, 2, torch.device("cpu"))))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_with_two_gloo_ranks():
    import socket

    import torch.multiprocessing as mp

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_max_worker, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: 3.5, 1: 3.5}
    assert bench._max_over_ranks(2.25, 1, None) == 2.25


def test_reference_arm_on_a_non_zero_rank_is_silent(built):
    import os

    env = dict(os.environ, WORLD_SIZE="2", RANK="1", LOCAL_RANK="1")
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference",
                          "--size", "32", "--steps", "1", "--warmup", "0"],
                         cwd=ROOT, capture_output=True, text=True, timeout=300, env=env)
    assert out.returncode == 0, out.stderr[-2000:]
    assert out.stdout.strip() == ""
