"""The multi-GPU path is independent replicas; its only host-side exchange is
bench.aggregate's max-over-ranks of the timed region.  Two gloo ranks on the
CPU check it (no GPU involved)."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import os, sys
sys.path.insert(0, sys.argv[1])
import torch.distributed as dist
import bench
dist.init_process_group("gloo")
rank = dist.get_rank()
# each rank opens its own GPU: the launcher's LOCAL_RANK among all visible
# devices, whatever CUDA_VISIBLE_DEVICES lists
assert bench.rank_device() == (rank if os.environ.get("VIS_MODE") != "one" else 0), bench.rank_device()
devs = [None, None]
dist.all_gather_object(devs, bench.rank_device())
if os.environ.get("VIS_MODE") != "one":
    assert devs == [0, 1], devs
total, value = bench.aggregate(100.0 * (rank + 1), 10, 5, dist)
assert total == 200.0, total
assert abs(value - 10 * 5 * 2 / 0.2) < 1e-9, value
dist.destroy_process_group()
print("ok", rank)
"""


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


@pytest.mark.parametrize("vis", ["unset", "all", "one"])
def test_two_gloo_replicas_take_the_slowest_time(vis):
    """vis: CUDA_VISIBLE_DEVICES unset, listing every GPU, or narrowed to
    this rank's one GPU by the launcher."""
    pytest.importorskip("torch.distributed")
    port = _free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), LOCAL_RANK=str(r), VIS_MODE=vis)
        env.pop("CUDA_VISIBLE_DEVICES", None)
        if vis == "all":
            env["CUDA_VISIBLE_DEVICES"] = "0,1,2,3,4,5,6,7"
        elif vis == "one":
            env["CUDA_VISIBLE_DEVICES"] = str(r)
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD, ROOT], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=120) for p in procs]
    for p, (o, e) in zip(procs, outs):
        assert p.returncode == 0, e
        assert o.startswith("ok")
