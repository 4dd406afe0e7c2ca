"""The bench's multi-process plumbing on CPU: two gloo ranks (world size 2).

The timed region of bench.py is bracketed by a barrier on every rank and
reports the maximum over ranks; under torchrun the reference arm runs on
rank 0 only and the other ranks leave without work.  These tests run those
helpers as two spawned processes that rendezvous on 127.0.0.1.
"""
import importlib.util
import io
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _load_bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    bench = _load_bench()

    class A:
        impl = "reference"

    w, r, local, pg = bench.dist_setup(A)
    assert (w, r, local) == (world, rank, rank) and pg is not None
    bench.barrier(pg)
    # each rank reports a different time; every rank must see the maximum
    got = bench.max_over_ranks(10.0 + 7.0 * rank, pg)
    bench.barrier(pg)
    pg.destroy_process_group()
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        f.write(repr(got))


def test_barrier_and_max_over_ranks_gloo(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    vals = [float(open(tmp_path / f"rank{r}.txt").read()) for r in range(world)]
    assert vals == [17.0, 17.0]


def _reference_rank(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    bench = _load_bench()
    if rank == 0:
        # rank 0 would run the CPU reference; here it only joins and leaves
        w, r, _, pg = bench.dist_setup(type("A", (), {"impl": "reference"}))
        pg.destroy_process_group()
        text = ""
    else:
        sys.argv = ["bench.py", "--impl", "reference", "--gpus", str(world)]
        args = bench.parse()
        buf = io.StringIO()
        with redirect_stdout(buf):
            bench.run_reference(args)
        text = buf.getvalue()
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        f.write(text)


def test_reference_arm_runs_on_rank_zero_only(tmp_path):
    """A rank other than 0 prints nothing and exits without work."""
    mp = pytest.importorskip("torch.multiprocessing")
    world = 2
    mp.spawn(_reference_rank, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    assert open(tmp_path / "rank1.txt").read() == ""
