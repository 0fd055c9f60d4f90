"""Shape pairs of the headline pile generator, for the narrowphase
cross-checks: settled worlds (the FP64 oracle advances them 300 env-steps),
every sphere-box and box-box pair whose bounding spheres come within 1 cm.
Poses are (x, y, z, qx, qy, qz, qw); pile geoms sit at their body's origin."""
import numpy as np

import oracle_py
from tooling_gb300 import scenes

SPHERE, BOX = 1, 2


def settled_pairs(n_worlds=64, first_world=500, steps=300):
    b = scenes.pile_batch(n_worlds=n_worlds, first_world=first_world)
    rq, _ = oracle_py.run(b, np.arange(len(b)), b.qpos, b.qvel, None, steps, precision=1, n_threads=8)
    gofs = np.concatenate([[0], np.cumsum(b.n_geoms)])
    sb, bb = [], []
    for w in range(len(b)):
        q = rq[b.q_off[w]:b.q_off[w] + b.nq[w]].reshape(-1, 7)
        g = b.geoms[gofs[w]:gofs[w + 1]]
        items = []
        for gg in g:
            if gg["body"] < 0:
                continue
            k = int(gg["body"])
            pose = np.r_[q[k, :3], q[k, 4:7], q[k, 3]].astype(np.float32)  # MuJoCo wxyz -> xyzw
            items.append((int(gg["shape"]), pose, np.array(gg["size"], np.float32)))
        for i, (si, pi, zi) in enumerate(items):
            for j, (sj, pj, zj) in enumerate(items):
                if i == j or np.linalg.norm(pi[:3] - pj[:3]) > np.linalg.norm(zi) + np.linalg.norm(zj) + 0.01:
                    continue
                if si == SPHERE and sj == BOX:
                    sb.append((pi, zi, pj, zj))
                elif si == BOX and sj == BOX and i < j:
                    bb.append((pi, zi, pj, zj))
    return sb, bb
