"""Seeded synthetic workloads (meshes in the reference's JSON format plus refinement scripts).

No public benchmark suite exists for this path; these generators produce the mesh families of the
five configurations the GPU path is measured on. A workload is a mesh JSON plus a list of operations
(the reference's Mesh API calls) so the same script can be replayed on any implementation:

    ("orders", i, j, ids|None)     set_global_expansion_orders / set_expansion_on_elems
    ("pref", di, dj, ids|None)     global_p_refinement / p_refine_elems
    ("href", kind, ids|None, ext)  global_h_refinement / h_refine_elems (kind 0 T, 1 U, 2 V)
    ("hmix", ids, kinds)           execute_h_refinements with one kind per Elem

Random choices use splitmix64 (seeded, identical on every machine); leaf sets are read back from the
mesh after each round, so a script is built against a mesh as it is refined. The mesh a script is
built on is a ``replay`` class: ``NativeReplay`` (this package's Mesh, the default) or any class with
the same three members (the oracle's ``OracleReplay``); both give the same script, so a caller that
must not load this package's library can still build every workload.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

MASK = (1 << 64) - 1


class SplitMix64:
    def __init__(self, seed):
        self.s = (int(seed) * 0x9E3779B97F4A7C15 + 0x1234567) & MASK

    def next(self):
        self.s = (self.s + 0x9E3779B97F4A7C15) & MASK
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK
        return z ^ (z >> 31)

    def uniform(self):
        return (self.next() >> 11) / float(1 << 53)

    def randint(self, lo, hi):
        """integer in [lo, hi] inclusive"""
        return lo + self.next() % (hi - lo + 1)

    def sample(self, items, k):
        """k distinct items, uniformly without replacement (partial Fisher-Yates), in drawn order"""
        items = list(items)
        k = min(k, len(items))
        for i in range(k):
            j = i + self.next() % (len(items) - i)
            items[i], items[j] = items[j], items[i]
        return items[:k]


def grid_mesh_json(nx, ny, x0, x1, y0, y1, materials=(1.0, 0.0, 1.0, 0.0)):
    """nx x ny quad Elems on [x0,x1]x[y0,y1]; node (i, j) has id j*(nx+1)+i (mesh.rs:100-141 format)."""
    xs = np.linspace(x0, x1, nx + 1)
    ys = np.linspace(y0, y1, ny + 1)
    nodes = [[float(x), float(y)] for y in ys for x in xs]
    els = []
    for j in range(ny):
        for i in range(nx):
            n0 = j * (nx + 1) + i
            els.append({"materials": list(materials), "node_ids": [n0, n0 + 1, n0 + nx + 1, n0 + nx + 2]})
    return {"Elements": els, "Nodes": nodes}


@dataclass
class Workload:
    name: str
    mesh_json: dict
    ops: list = field(default_factory=list)
    basis: int = 0            # 0 HierPoly, 1 KOLeg
    glq: tuple = (8, 8)
    target: float = 10.0
    n_pairs: int = 1
    seed: int = 0
    note: str = ""


def apply_ops(mesh, ops):
    """Replay a script on a fem_2d_gb300.Mesh."""
    from . import Orders, PRef

    for op in ops:
        if op[0] == "orders":
            _, i, j, ids = op
            if ids is None:
                mesh.set_global_expansion_orders(Orders(i, j))
            else:
                mesh.set_expansion_on_elems(ids, Orders(i, j))
        elif op[0] == "pref":
            _, di, dj, ids = op
            if ids is None:
                mesh.global_p_refinement(PRef(di, dj))
            else:
                mesh.p_refine_elems(ids, PRef(di, dj))
        elif op[0] == "href":
            _, kind, ids, ext = op
            if ids is None:
                mesh.global_h_refinement((kind, ext))
            else:
                mesh.h_refine_elems(ids, (kind, ext))
        elif op[0] == "hmix":
            _, ids, kinds = op
            mesh.execute_h_refinements([(e, (k, -1)) for e, k in zip(ids, kinds)])
        elif op[0] == "ordersmap":
            _, table = op
            for (i, j), ids in table:
                mesh.set_expansion_on_elems(ids, Orders(i, j))
        else:
            raise ValueError(op[0])


class NativeReplay:
    """A script under construction replayed on this package's Mesh."""

    def __init__(self, mesh_json):
        from . import Mesh

        self.mesh = Mesh.from_json(mesh_json)

    def apply(self, ops):
        apply_ops(self.mesh, ops)

    def elem_info(self):
        """Per Elem: [is_leaf, ni, nj, parent, nodes(4), edges(4), h_u, h_v]."""
        return self.mesh.elem_info()


def _leaves(mesh):
    info = mesh.elem_info()
    return [int(e) for e in np.nonzero(info[:, 0] == 1)[0]]


def _random_rounds(mesh, ops, rng, rounds, fraction, kinds):
    for _ in range(rounds):
        leaves = _leaves(mesh)
        pick = sorted(rng.sample(leaves, int(fraction * len(leaves))))
        ks = [kinds[rng.next() % len(kinds)] for _ in pick]
        op = ("hmix", pick, ks)
        mesh.apply([op])
        ops.append(op)


def waveguide_small(replay=NativeReplay):
    """[0,1]x[0,0.5] in 2 Elems, orders (4,4), global T, then U on the leaves touching the top-middle node
    (the README.md:45-61 sequence); HierPoly, GLQ [8,8], dense solve nearest 10.0 (TE10: pi^2)."""
    mj = grid_mesh_json(2, 1, 0.0, 1.0, 0.0, 0.5)
    ops = [("orders", 4, 4, None), ("href", 0, None, -1)]
    m = replay(mj)
    m.apply(ops)
    info = m.elem_info()
    center = int(info[0, 4 + 3])   # elems[0].nodes[3]
    pick = [e for e in range(len(info)) if info[e, 0] == 1 and center in info[e, 4:8]]
    ops.append(("href", 1, pick, -1))
    return Workload("waveguide_small", mj, ops, basis=0, glq=(8, 8), target=10.0, n_pairs=1)


def precision(seed=0, nx=16, ny=8, order=6, rounds=3, fraction=0.3, replay=NativeReplay):
    """[0,2]x[0,1], 16x8 Elems, orders (6,6), three seeded rounds refining 30% of the leaves with T/U/V;
    KOLeg, GLQ [10,10], 10 pairs nearest 10.0."""
    mj = grid_mesh_json(nx, ny, 0.0, 2.0, 0.0, 1.0)
    ops = [("orders", order, order, None)]
    m = replay(mj)
    m.apply(ops)
    _random_rounds(m, ops, SplitMix64(seed), rounds, fraction, [0, 1, 2])
    return Workload("precision_16x8_p6_koleg", mj, ops, basis=1, glq=(10, 10), target=10.0, n_pairs=10, seed=seed)


def full_scale(seed=0, nx=64, ny=32, rounds=4, fraction=0.3, pmin=3, pmax=8, basis=0, replay=NativeReplay):
    """[0,2]x[0,1], 64x32 Elems, per-Elem orders uniform in pmin..pmax per direction, `rounds` seeded rounds
    of T/U/V refinement of `fraction` of the leaves; HierPoly (basis=0) or KOLeg (basis=1), GLQ [10,10],
    20 pairs nearest 10.0."""
    mj = grid_mesh_json(nx, ny, 0.0, 2.0, 0.0, 1.0)
    rng = SplitMix64(seed)
    groups = {}
    for e in range(nx * ny):
        key = (rng.randint(pmin, pmax), rng.randint(pmin, pmax))
        groups.setdefault(key, []).append(e)
    ops = [("ordersmap", sorted(groups.items()))]
    m = replay(mj)
    m.apply(ops)
    _random_rounds(m, ops, rng, rounds, fraction, [0, 1, 2])
    name = "full_%dx%d_p%d-%d_%s_r%d_f%g" % (nx, ny, pmin, pmax, "koleg" if basis else "hierpoly", rounds, fraction)
    return Workload(name, mj, ops, basis=basis, glq=(10, 10), target=10.0, n_pairs=20, seed=seed)


def learned_family(seed=0, nx=32, ny=16, orders=(5, 7), rounds=2, fraction=1.0, replay=NativeReplay):
    """The learned-preconditioner family: [0,2]x[0,1], nx x ny Elems, orders (5,7), `rounds` seeded rounds of
    anisotropic (U/V) refinement of `fraction` of the leaves (two rounds from a uniform grid keep Elems that
    share an edge within two levels); KOLeg, GLQ [10,10], 10 pairs nearest 10.0. Full size 32x16."""
    mj = grid_mesh_json(nx, ny, 0.0, 2.0, 0.0, 1.0)
    ops = [("orders", orders[0], orders[1], None)]
    m = replay(mj)
    m.apply(ops)
    _random_rounds(m, ops, SplitMix64(7919 * (seed + 1)), rounds, fraction, [1, 2])
    return Workload("learned_%dx%d_p%d-%d_seed%d" % (nx, ny, orders[0], orders[1], seed), mj, ops, basis=1,
                    glq=(10, 10), target=10.0, n_pairs=10, seed=seed)


def batch_member(seed, replay=NativeReplay):
    """One mesh of the batching family: a ~ U[1,3], (gx, gy) with gx*gy in [4,64] on [0,a]x[0,1],
    per-Elem orders (pu, pv) ~ U{2..8}^2, 0-2 random refinement rounds; GLQ [10,10], 4 pairs nearest 10."""
    rng = SplitMix64(1000003 * (seed + 1))
    a = 1.0 + 2.0 * rng.uniform()
    while True:
        gx, gy = rng.randint(1, 16), rng.randint(1, 8)
        if 4 <= gx * gy <= 64:
            break
    mj = grid_mesh_json(gx, gy, 0.0, a, 0.0, 1.0)
    groups = {}
    for e in range(gx * gy):
        groups.setdefault((rng.randint(2, 8), rng.randint(2, 8)), []).append(e)
    ops = [("ordersmap", sorted(groups.items()))]
    m = replay(mj)
    m.apply(ops)
    _random_rounds(m, ops, rng, rng.randint(0, 2), 0.3, [0, 1, 2])
    return Workload("batch_%d" % seed, mj, ops, basis=0, glq=(10, 10), target=10.0, n_pairs=4, seed=seed)


def build_mesh(w):
    from . import Mesh

    m = Mesh.from_json(w.mesh_json)
    apply_ops(m, w.ops)
    return m
