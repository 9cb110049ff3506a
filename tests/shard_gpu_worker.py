"""One rank of the sharded GPU gradient test: the exact gradient of a share of
the shots of a small PSV problem, computed by a Sim on the GPU (forward
operator, misfit, reverse sweep; the Sim sums its shots in FP32), then the
rank-ordered sum of the ranks' fields (seiswg_gb300.shards.reduce_gradients,
gloo on host tensors).  With WORLD = 1 and no port it computes every shot in
one process, the reference the test compares with.

    python tests/shard_gpu_worker.py RANK WORLD PORT OUT.npz
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import seiswg_gb300 as sw  # noqa: E402
from seiswg_gb300 import shards  # noqa: E402

NX, NZ, NT, DX, DT = 160, 200, 400, 10.0, 1.2e-3
SHOTS = [(30, 20), (60, 20), (90, 20), (120, 20), (75, 40)]
PARAMS = ("lambda", "mu", "buoyancy")


def _sim(vp_scale):
    rng = np.random.default_rng(5)
    vp = (3000 * (1 + 0.04 * np.tanh(rng.standard_normal((NX, NZ))))).astype(np.float32) * np.float32(vp_scale)
    sim = sw.Sim(NX, NZ, NT, DX, DX, DT, psv=True, abs_left=True, abs_right=True, abs_bottom=True, abs_width=12)
    sim.upload_model("vp", vp)
    sim.upload_model("vs", (vp / np.sqrt(3)).astype(np.float32))
    sim.upload_model("rho", np.full((NX, NZ), 2500.0, np.float32))
    sim.prepare()
    stf = np.stack([sw.ricker(NT, DT, 20.0, 0.06, 30.0 + 10 * k, 1.0e10) for k in range(len(SHOTS))], axis=1)
    sim.set_sources([s[0] for s in SHOTS], [s[1] for s in SHOTS], stf)
    rec = list(range(8, NX - 8, 6))
    sim.set_receivers(rec, [100] * len(rec))
    return sim


def local_sum(units):
    """The Sim's own sum over `units` of the shot gradients (uninverted
    parameters lambda, mu, buoyancy)."""
    true = _sim(1.03)
    obs = {}
    for k in units:
        true.forward(k)
        obs[k] = true.traces()[[0, 2]]
    true.close()
    sim = _sim(1.0)
    sim.gradient_clear()
    for k in units:
        sim.forward_op(k, 0)
        _, adj = sw.l2_misfit(sim.traces()[[0, 2]], obs[k], DT)
        sim.backward_op(adj)
    g = {p: sim.gradient(p) for p in PARAMS}
    sim.close()
    return g


def main():
    rank, world, port, out = int(sys.argv[1]), int(sys.argv[2]), sys.argv[3], sys.argv[4]
    if world == 1:
        np.savez(out, units=np.arange(len(SHOTS)), **local_sum(range(len(SHOTS))))
        return
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = shards.my_units([1.0] * len(SHOTS), rank, world)
        total = shards.reduce_gradients(local_sum(mine))
        np.savez(out if rank == 0 else out + f".r{rank}", units=np.array(mine), **total)
    finally:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
