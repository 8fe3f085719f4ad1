"""Frequency sharding of bench.py over ranks (the multi-GPU form of the path:
frequencies are independent units, so each rank solves its own share with no
data-path collective; the only exchange is the max over ranks of the timing).

Two CPU ranks on the gloo backend run bench.py's sharding and timing logic with
a stub solver in place of the GPU library.  Not measured on GPU hardware: every
GPU machine of this build has one GPU."""
import json
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, steps, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    my = bench.shard(bench.OMEGAS, rank, world)
    seen = []

    def stub(oms):
        # a solver whose device span differs per rank: rank r takes (r + 1) * 40 ms
        seen.extend(float(o) for o in oms)
        return 40.0 * (rank + 1), {"n": len(oms)}

    r = bench.timed_sweep(stub, my, steps, dist, world)
    with open(os.path.join(out_dir, "rank%d.json" % rank), "w") as f:
        json.dump({"my": [float(x) for x in my], "timed": [float(x) for x in r["timed"]], "seen": seen,
                   "dev_ms": r["dev_ms"], "dev_ms_max": r["dev_ms_max"], "value": r["value"],
                   "wall_max": r["wall_max"], "e2e": r["e2e"]}, f)
    dist.destroy_process_group()


@pytest.mark.parametrize("world,steps", [(2, 20), (2, 3)])
def test_two_rank_sharding_and_max_timing(tmp_path, world, steps):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(world, port, steps, str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    sys.path.insert(0, ROOT)
    import bench
    out = [json.load(open(tmp_path / ("rank%d.json" % r))) for r in range(world)]
    shares = [set(o["my"]) for o in out]
    # the shares are disjoint and together are the whole sweep
    assert not (shares[0] & shares[1])
    assert sorted(shares[0] | shares[1]) == sorted(float(x) for x in bench.OMEGAS)
    for o, sh in zip(out, shares):
        # each rank solved exactly its timed frequencies, all from its own share
        assert o["seen"] == o["timed"] and len(o["timed"]) == steps
        assert set(o["timed"]) <= sh
        # the whole-job value divides every rank's frequency-solves by the slowest rank's device time
        assert o["dev_ms_max"] == pytest.approx(40.0 * world)
        assert o["value"] == pytest.approx(steps * world / (40.0 * world / 1000.0))
        assert o["e2e"] == pytest.approx(steps * world / o["wall_max"])
    # every rank reports the same max
    assert len({o["dev_ms_max"] for o in out}) == 1 and len({o["wall_max"] for o in out}) == 1
    # the timed frequencies spread over the sweep: lowest and highest quarter both represented
    if steps >= 8:
        for o in out:
            t = np.array(o["timed"])
            assert t.min() < 0.8 and t.max() > 2.2
