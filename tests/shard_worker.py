"""One rank of the sharded-gradient test: a share of the shots of a small PSV
problem (FP64 oracle exact gradients, summed in FP32 per rank as a Sim's
accumulator does), then the rank-ordered sum across ranks.

    python tests/shard_worker.py RANK WORLD PORT OUT.npz
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from seiswg_gb300 import shards  # noqa: E402

NX, NZ, NT, DX, DT = 30, 36, 120, 10.0, 1.5e-3
SHOTS = [(6, 12), (12, 12), (18, 12), (24, 12), (15, 20)]


def problem():
    s = O.Setup(NX, NZ, NT, DX, DX, DT, sh=False, psv=True, abs_left=True, abs_bottom=True, abs_width=6)
    rng = np.random.default_rng(3)
    vp = 3000 * (1 + 0.04 * rng.standard_normal((NX, NZ)))
    vs = vp / np.sqrt(3)
    rho = np.full((NX, NZ), 2500.0)
    src = [i * NZ + j for i, j in SHOTS]
    stf = O.stf_table([(0, 0, 25.0, 0.04, 30.0 + 10 * k, 1e10) for k in range(len(SHOTS))], NT, DT, 64)
    rec = np.array([i * NZ + 4 for i in range(2, NX - 2, 3)], np.int32)
    return s, vp, vs, rho, src, stf, rec


def shot_gradient(k, model=None):
    s, vp, vs, rho, src, stf, rec = problem()

    def run(vp_):
        o = O.FD2DOracle(s, src, stf, rec, 64)
        o.set_field("LAM", vp_)
        o.set_field("MU", vs)
        o.set_field("RHO", rho)
        o.init_model()
        o.run_forward(k)
        return o, np.stack([o.obs("X"), o.obs("Z")])

    _, obs = run(vp * 1.03)
    o, syn = run(vp)
    _, adj = O.l2_misfit(syn, obs, DT)
    gl, gm, gb = o.exact_gradient(adj, k)
    return {"lambda": gl.astype(np.float32), "mu": gm.astype(np.float32), "buoyancy": gb.astype(np.float32)}


def local_sum(units):
    acc = {n: np.zeros((NX, NZ), np.float32) for n in ("lambda", "mu", "buoyancy")}
    for k in units:
        g = shot_gradient(k)
        for n in acc:
            acc[n] += g[n]
    return acc


def main():
    rank, world, port, out = int(sys.argv[1]), int(sys.argv[2]), sys.argv[3], sys.argv[4]
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        costs = [1.0] * len(SHOTS)
        mine = shards.my_units(costs, rank, world)
        total = shards.reduce_gradients(local_sum(mine))
        if rank == 0:
            np.savez(out, units=np.array(mine), **total)
        else:
            np.savez(out + f".r{rank}", units=np.array(mine), **total)
    finally:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
