"""The small scenes used to compare renders with the reference's own CUDA renderer:
the 2x2x2-block seeded workload (depths 3-4, 10% masked nodes, 160x120) with its
default transfer function ("default"), a constant colour/opacity transfer
function that isolates the masking and sample-count behaviour ("const"), and a
field linear in the world coordinates with no masked nodes ("linear")."""
from __future__ import annotations

import numpy as np

from revise_gb300 import workloads

VARIANTS = ("default", "const", "linear")


def workload(variant: str):
    w = workloads.small(seed=2, level=1, depths=(3, 4), W=160, H=120, mask_fraction=0.1)
    if variant == "const":
        w.tf = np.tile(np.array([[0.8, 0.4, 0.2, 0.3]], np.float32), (256, 1))
    elif variant == "linear":
        for b in range(w.nblocks):
            a, c = int(w.node_off[b]), int(w.node_off[b + 1])
            u = w.n2i[a:c].astype(np.float64) / (1 << int(w.blocks[b, 3])) + w.blocks[b, :3]
            w.sparse[a:c] = (0.25 * u[:, 0] + 0.2 * u[:, 1] + 0.1 * u[:, 2]).astype(np.float32)
        w.field_min, w.field_max = 0.0, 1.1
    w.tf = np.ascontiguousarray(w.tf, dtype=np.float32)
    return w


def b2f_blocks(w):
    """Block rows of w in back-to-front order for its eye."""
    from revise_gb300 import host
    m = 1 << w.level
    order = host.b2f_order([0, 0, 0], [m, m, m], [-5.0] * 3, [5.0] * 3, w.eye)
    idx = {tuple(b[:3]): i for i, b in enumerate(w.blocks.tolist())}
    return [idx[tuple(b)] for b in order.tolist()]
