"""bench.py's multi-GPU path is N independent replicas (one process per GPU,
no collective on the data path): the timing is the maximum over ranks and
the whole-job rate counts every replica's cells.  Checked here with two
gloo ranks on the CPU, through the same helpers the bench uses; the
reference arm runs on rank 0 alone."""

import json
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(WORLD_SIZE=str(world), RANK=str(rank), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench._max_over_ranks(10.0 * (rank + 1), "cpu")
        rate = bench._whole_job_rate(1000, 4, ms)
        ref = None
        if rank != 0:
            # the reference arm: ranks other than 0 return without work
            class A:
                steps = 1
                warmup = 1
            ref = bench.run_reference(A())
        with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
            json.dump({"ms": ms, "rate": rate, "ref": ref}, f)
    finally:
        dist.destroy_process_group()


def test_replicas_time_is_max_over_ranks_and_rate_counts_every_replica(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    for r in range(world):
        d = json.loads((tmp_path / f"rank{r}.json").read_text())
        assert d["ms"] == 20.0
        assert d["rate"] == pytest.approx(1000 * 4 * world / 0.020)
        assert d["ref"] is None


def test_reference_arm_prints_the_contract_line(capsys, monkeypatch):
    """`bench.py --impl reference` on rank 0: one JSON line with the metric,
    impl "reference", its CPU baseline and an end-to-end figure without host
    copies (small domain here; the bench runs the full workload)."""
    import bench

    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    # the arm sets these only where unset; set here, they are restored afterwards
    monkeypatch.setenv("OMP_NUM_THREADS", "1")
    monkeypatch.setenv("GETM_ORACLE_VARIANT", "serial")
    monkeypatch.setattr("sys.argv", ["bench.py", "--impl", "reference", "--nx", "24", "--ny", "20", "--nz", "4",
                                     "--steps", "1", "--warmup", "1"])
    bench.main()
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["metric"] == "3D cell-updates/s"
    assert line["value"] > 0 and line["higher_is_better"] is True
    assert line["cpu_baseline"]["value"] == line["value"] and line["cpu_baseline"]["kind"] == "port"
    assert line["cpu_baseline"]["cores"] == 1  # the threads it ran with
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["steps"] == 1 and line["warmup"] == 1
    # the same workload description as the GPU arm prints
    from getm_gb300 import workloads

    assert line["config"] == bench._config(workloads.seamount(nx=24, ny=20, nz=4), 1)
