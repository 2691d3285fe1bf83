"""Quadtree / octree mesh hierarchy and its flat neighbour tables.

ThunderEgg builds its level hierarchy from a p4est/p8est forest
(P4estDomainGenerator.cpp:205-738, P8estDomainGenerator.cpp).  p4est is not a
dependency here, so this module re-creates the same semantics on a single
tree covering the unit square / cube:

* leaves of the finest level are ordered in Morton (z) order, x fastest, and
  get ids 0..N-1 in that order (SetIds, P4estDomainGenerator.cpp:170-189);
* each coarser level coarsens every complete family whose level is above the
  new level; the coarse patch takes the id of its first (south-west) child and
  lists its children by orthant; the children get ``parent_id`` = that id and
  ``orth_on_parent`` = their orthant.  Patches that are not coarsened point to
  themselves with ``orth_on_parent`` = null (coarsenTree, :272-321);
* face neighbours are Normal / Coarse (with the orthant of this patch on the
  coarse face) / Fine (ids ordered by orthant on the face)
  (addCoarseNbrInfo/addFineNbrInfo/addNormalNbrInfo, :374-470);
* corner (and in 3D edge) neighbours exist only where the corner / edge is a
  corner / edge of every leaf around it (p4est's corner and edge iterators,
  :606-640, P8estDomainGenerator.cpp:812-850); a coarse corner neighbour has
  orth_on_coarse = 0, a coarse edge neighbour the half of the coarse edge.

The result is a list of :class:`MeshLevel` (finest first) whose arrays are
exactly the ``te_level_desc`` tables of ``include/te_gpu.h``.
"""
from __future__ import annotations

import ctypes
import itertools
import json
import dataclasses
import math
from dataclasses import dataclass, field

import numpy as np

NBR_NONE, NBR_NORMAL, NBR_COARSE, NBR_FINE = -1, 0, 1, 2


# ---------------------------------------------------------------------------
# face indexing (Face.h:41-125, 558-584)
# ---------------------------------------------------------------------------
def num_face_slots(dim: int) -> int:
    return 8 if dim == 2 else 26


def side_slot(dim: int, side: int) -> int:
    """slot of Side<D>(side) in PatchInfo::nbr_infos"""
    return (4 if dim == 2 else 20) + side


def corner_slot(dim: int, corner: int) -> int:
    return corner


def edge_slot(edge: int) -> int:
    return 8 + edge


def tangential_axes(dim: int, axis: int):
    return [a for a in range(dim) if a != axis]


def edge_axes(edge: int):
    """Edge value -> (parallel axis, (t0, t1), (upper0, upper1))  (Face.h:405-480)."""
    axis = edge >> 2
    t = [a for a in range(3) if a != axis]
    return axis, t, ((edge >> 0) & 1, (edge >> 1) & 1)


def make_edge(axis: int, upper0: int, upper1: int) -> int:
    return (axis << 2) | upper0 | (upper1 << 1)


def opposite_face(dim: int, m: int, value: int) -> int:
    """Face<D,M>::opposite (Face.h:490): flip the D-M side bits."""
    return value ^ ((1 << (dim - m)) - 1)


# ---------------------------------------------------------------------------
# leaves
# ---------------------------------------------------------------------------
Leaf = tuple  # (level, (i, j[, k]))


def uniform_leaves(dim: int, level: int):
    m = 1 << level
    return {(level, c) for c in itertools.product(range(m), repeat=dim)}


def _children(dim, leaf):
    l, c = leaf
    out = []
    for o in range(1 << dim):
        out.append((l + 1, tuple(2 * c[a] + ((o >> a) & 1) for a in range(dim))))
    return out


def refine_leaves(leaves, dim: int, pred, lo: int, hi: int):
    """Refine, level by level from ``lo`` to ``hi - 1``, every leaf of that
    level for which ``pred(level, coords)`` is true."""
    leaves = set(leaves)
    for l in range(lo, hi):
        nxt = set()
        for leaf in sorted(leaves):
            if leaf[0] == l and pred(*leaf):
                nxt.update(_children(dim, leaf))
            else:
                nxt.add(leaf)
        leaves = nxt
    return leaves


def circle_intersects(level, c, r=0.3, cx=0.5, cy=0.5):
    """Leaf box meets the circle *curve* |x - (cx, cy)| = r."""
    h = 1.0 / (1 << level)
    x0, y0 = c[0] * h, c[1] * h
    dx = max(x0 - cx, 0.0, cx - (x0 + h))
    dy = max(y0 - cy, 0.0, cy - (y0 + h))
    dmin = math.hypot(dx, dy)
    dmax = max(math.hypot(x - cx, y - cy) for x in (x0, x0 + h) for y in (y0, y0 + h))
    return dmin <= r <= dmax


def circle_leaves(lo=3, hi=7, r=0.3, center=(0.5, 0.5)):
    leaves = uniform_leaves(2, lo)
    return refine_leaves(leaves, 2, lambda l, c: circle_intersects(l, c, r, *center), lo, hi)


def random_leaves(seed: int, dim=2, lo=2, hi=6, p=0.3):
    """Each leaf refined with probability p, level by level from lo up to hi."""
    rng = np.random.default_rng(seed)
    leaves = uniform_leaves(dim, lo)
    for l in range(lo, hi):
        nxt = set()
        for leaf in sorted(leaves):
            if leaf[0] == l and rng.random() < p:
                nxt.update(_children(dim, leaf))
            else:
                nxt.add(leaf)
        leaves = nxt
    return leaves


class _LeafIndex:
    def __init__(self, leaves, dim):
        self.dim = dim
        self.set = set(leaves)
        self.maxl = max(l for l, _ in leaves)

    def covering(self, level, c):
        """Leaf containing cell c of ``level`` (level <= that of the cell), or
        None when the cell is subdivided / outside the domain."""
        m = 1 << level
        leaves = self.set
        if len(c) == 2:
            x, y = c
            if x < 0 or y < 0 or x >= m or y >= m:
                return None
            for L in range(level, -1, -1):
                key = (L, (x, y))
                if key in leaves:
                    return key
                x >>= 1
                y >>= 1
            return None
        for x in c:
            if x < 0 or x >= m:
                return None
        cc = tuple(c)
        for L in range(level, -1, -1):
            key = (L, cc)
            if key in leaves:
                return key
            cc = tuple(x >> 1 for x in cc)
        return None

    def leaf_at_point(self, p):
        """Leaf containing the finest-resolution cell p (coords at maxl)."""
        return self.covering(self.maxl, p)


def balance_leaves(leaves, dim: int, connect: str = "full"):
    """2:1 balance across faces (connect='face') or faces, edges and corners
    (connect='full'), as p4est_balance with P4EST_CONNECT_FACE / FULL."""
    leaves = set(leaves)
    if connect == "face":
        dirs = [tuple((1 if b == a else 0) * s for b in range(dim))
                for a in range(dim) for s in (-1, 1)]
    else:
        dirs = [d for d in itertools.product((-1, 0, 1), repeat=dim) if any(d)]
    changed = True
    while changed:
        changed = False
        idx = _LeafIndex(leaves, dim)
        split = set()
        for (l, c) in leaves:
            for d in dirs:
                nc = tuple(c[a] + d[a] for a in range(dim))
                q = idx.covering(l, nc)
                if q is not None and q[0] < l - 1:
                    split.add(q)
        if split:
            changed = True
            for q in split:
                leaves.discard(q)
                leaves.update(_children(dim, q))
    return leaves


def morton_key(dim, leaf, maxl):
    l, c = leaf
    s = maxl - l
    key = 0
    anchors = [x << s for x in c]
    for bit in range(maxl):
        for a in range(dim):
            key |= ((anchors[a] >> bit) & 1) << (bit * dim + a)
    return (key, l)


# ---------------------------------------------------------------------------
# level tables
# ---------------------------------------------------------------------------
@dataclass
class MeshLevel:
    """One Domain<D>: the flattened PatchInfo<D> vector (PatchInfo.h:66-126)."""

    dim: int
    ns: tuple
    num_ghost: int
    id: np.ndarray
    refine_level: np.ndarray
    parent_id: np.ndarray
    orth_on_parent: np.ndarray
    child_ids: np.ndarray
    starts: np.ndarray
    spacings: np.ndarray
    nbr_type: np.ndarray
    nbr_ids: np.ndarray
    nbr_orth: np.ndarray
    quads: list = field(default_factory=list)  # (level, coords) per patch, if known
    _keep: list = field(default_factory=list, repr=False)

    @property
    def num_patches(self):
        return int(self.id.shape[0])

    @property
    def cells_per_patch(self):
        return int(np.prod(self.ns[: self.dim]))

    @property
    def num_cells(self):
        return self.num_patches * self.cells_per_patch

    def padded_shape(self, ncomp=1):
        g = self.num_ghost
        sp = [self.ns[a] + 2 * g for a in range(self.dim)]
        return (self.num_patches, ncomp) + tuple(reversed(sp))

    def patch_stride(self, ncomp=1):
        return int(np.prod(self.padded_shape(ncomp)[1:]))

    def id_to_local(self):
        return {int(i): k for k, i in enumerate(self.id)}

    def has_nbr(self, p, slot):
        return self.nbr_type[p, slot] != NBR_NONE

    def to_desc(self):
        """ctypes te_level_desc pointing at (kept-alive) contiguous copies."""
        from .capi import TeLevelDesc

        arrs = {}
        for name, dt in (("id", np.int32), ("refine_level", np.int32), ("parent_id", np.int32),
                         ("orth_on_parent", np.int32), ("child_ids", np.int32),
                         ("starts", np.float64), ("spacings", np.float64),
                         ("nbr_type", np.int32), ("nbr_ids", np.int32), ("nbr_orth", np.int32)):
            arrs[name] = np.ascontiguousarray(getattr(self, name), dtype=dt)
        d = TeLevelDesc()
        d.dim = self.dim
        ns = list(self.ns) + [1] * (3 - len(self.ns))
        d.ns = (ctypes.c_int * 3)(*ns[:3])
        d.num_ghost = self.num_ghost
        d.num_patches = self.num_patches
        for name, a in arrs.items():
            ct = ctypes.c_double if a.dtype == np.float64 else ctypes.c_int
            setattr(d, name, a.ctypes.data_as(ctypes.POINTER(ct)))
        self._keep = [arrs, d]
        return d

    # -- JSON (json.cpp:160-300 format, as in the reference's test/mesh_inputs)
    @staticmethod
    def from_json_level(patches, dim, ns, num_ghost=1):
        return _level_from_json(patches, dim, ns, num_ghost)


def _empty_level(dim, P, ns, num_ghost):
    F = num_face_slots(dim)
    return MeshLevel(
        dim=dim, ns=tuple(ns), num_ghost=num_ghost,
        id=np.zeros(P, np.int32), refine_level=np.full(P, -1, np.int32),
        parent_id=np.full(P, -1, np.int32), orth_on_parent=np.full(P, -1, np.int32),
        child_ids=np.full((P, 1 << dim), -1, np.int32),
        starts=np.zeros((P, dim)), spacings=np.ones((P, dim)),
        nbr_type=np.full((P, F), NBR_NONE, np.int32), nbr_ids=np.full((P, F, 4), -1, np.int32),
        nbr_orth=np.full((P, F), -1, np.int32))


def _quad_bbox(leaf, maxl):
    l, c = leaf
    s = maxl - l
    lo = tuple(x << s for x in c)
    hi = tuple((x + 1) << s for x in c)
    return lo, hi


def _link_level(lvl: MeshLevel, quads, connect: str):
    """Fill nbr_type/nbr_ids/nbr_orth for the quads (one per patch) of lvl."""
    dim = lvl.dim
    idx = _LeafIndex(quads, dim)
    maxl = idx.maxl
    qid = {q: int(lvl.id[k]) for k, q in enumerate(quads)}
    boxes = {}

    def bbox(q):
        b = boxes.get(q)
        if b is None:
            b = boxes[q] = _quad_bbox(q, maxl)
        return b
    for p, (l, c) in enumerate(quads):
        # ---- sides
        for axis in range(dim):
            tang = tangential_axes(dim, axis)
            for upper in (0, 1):
                side = 2 * axis + upper
                slot = side_slot(dim, side)
                nc = list(c)
                nc[axis] += 1 if upper else -1
                nc = tuple(nc)
                if nc[axis] < 0 or nc[axis] >= (1 << l):
                    continue
                q = idx.covering(l, nc)
                if q is not None and q[0] == l:
                    lvl.nbr_type[p, slot] = NBR_NORMAL
                    lvl.nbr_ids[p, slot, 0] = qid[q]
                elif q is not None:
                    if q[0] != l - 1:
                        raise ValueError("mesh is not 2:1 balanced across faces")
                    lvl.nbr_type[p, slot] = NBR_COARSE
                    lvl.nbr_ids[p, slot, 0] = qid[q]
                    lvl.nbr_orth[p, slot] = sum((c[t] & 1) << i for i, t in enumerate(tang))
                else:
                    lvl.nbr_type[p, slot] = NBR_FINE
                    for o in range(1 << (dim - 1)):
                        fc = [0] * dim
                        fc[axis] = 2 * nc[axis] + (0 if upper else 1)
                        for i, t in enumerate(tang):
                            fc[t] = 2 * c[t] + ((o >> i) & 1)
                        f = (l + 1, tuple(fc))
                        if f not in qid:
                            raise ValueError("mesh is not 2:1 balanced across faces")
                        lvl.nbr_ids[p, slot, o] = qid[f]
        if connect != "full":
            continue
        lo, hi = bbox((l, c))
        # ---- corners: every leaf around the vertex has it as a corner
        for corner in range(1 << dim):
            v = tuple(hi[a] if (corner >> a) & 1 else lo[a] for a in range(dim))
            around = {}
            ok = True
            for d in itertools.product((0, 1), repeat=dim):
                pt = tuple(v[a] - 1 + d[a] for a in range(dim))
                q = idx.leaf_at_point(pt)
                if q is None:
                    ok = False
                    break
                qlo, qhi = bbox(q)
                for a in range(dim):
                    if (d[a] == 1 and qlo[a] != v[a]) or (d[a] == 0 and qhi[a] != v[a]):
                        ok = False
                around[d] = q
                if not ok:
                    break
            if not ok:
                continue
            # direction of the diagonal cell: across every axis from this patch
            ddir = tuple(1 if (corner >> a) & 1 else 0 for a in range(dim))
            q = around[ddir]
            slot = corner_slot(dim, corner)
            if q[0] == l:
                lvl.nbr_type[p, slot] = NBR_NORMAL
            elif q[0] < l:
                lvl.nbr_type[p, slot] = NBR_COARSE
                lvl.nbr_orth[p, slot] = 0
            else:
                lvl.nbr_type[p, slot] = NBR_FINE
            lvl.nbr_ids[p, slot, 0] = qid[q]
        if dim != 3:
            continue
        # ---- edges (3D)
        for edge in range(12):
            axis, (t0, t1), (u0, u1) = edge_axes(edge)
            v0 = hi[t0] if u0 else lo[t0]
            v1 = hi[t1] if u1 else lo[t1]
            # span of the edge: widen to the coarsest leaf touching this edge
            seg_lo, seg_hi = lo[axis], hi[axis]
            regions = {}
            ok = True
            for _ in range(2):
                regions = {}
                for d0 in (0, 1):
                    for d1 in (0, 1):
                        leaves_here = []
                        a = seg_lo
                        while a < seg_hi:
                            pt = [0, 0, 0]
                            pt[axis] = a
                            pt[t0] = v0 - 1 + d0
                            pt[t1] = v1 - 1 + d1
                            q = idx.leaf_at_point(tuple(pt))
                            if q is None:
                                ok = False
                                break
                            qlo, qhi = bbox(q)
                            if q not in leaves_here:
                                leaves_here.append(q)
                            a = qhi[axis]
                        if not ok:
                            break
                        regions[(d0, d1)] = leaves_here
                    if not ok:
                        break
                if not ok:
                    break
                # widen once to the largest leaf's extent along the axis
                nlo, nhi = seg_lo, seg_hi
                for qs in regions.values():
                    for q in qs:
                        qlo, qhi = bbox(q)
                        nlo, nhi = min(nlo, qlo[axis]), max(nhi, qhi[axis])
                if (nlo, nhi) == (seg_lo, seg_hi):
                    break
                seg_lo, seg_hi = nlo, nhi
            if not ok:
                continue
            for (d0, d1), qs in regions.items():
                for q in qs:
                    qlo, qhi = bbox(q)
                    if (d0 == 1 and qlo[t0] != v0) or (d0 == 0 and qhi[t0] != v0):
                        ok = False
                    if (d1 == 1 and qlo[t1] != v1) or (d1 == 0 and qhi[t1] != v1):
                        ok = False
            if not ok:
                continue
            slot = edge_slot(edge)
            # the diagonal region restricted to this patch's extent along the axis
            diag = [q for q in regions[(u0, u1)]
                    if bbox(q)[0][axis] < hi[axis]
                    and bbox(q)[1][axis] > lo[axis]]
            if len(diag) == 1 and diag[0][0] == l:
                lvl.nbr_type[p, slot] = NBR_NORMAL
                lvl.nbr_ids[p, slot, 0] = qid[diag[0]]
            elif len(diag) == 1 and diag[0][0] < l:
                lvl.nbr_type[p, slot] = NBR_COARSE
                lvl.nbr_ids[p, slot, 0] = qid[diag[0]]
                lvl.nbr_orth[p, slot] = c[axis] & 1
            else:
                lvl.nbr_type[p, slot] = NBR_FINE
                diag.sort(key=lambda q: bbox(q)[0][axis])
                for o, q in enumerate(diag[:2]):
                    lvl.nbr_ids[p, slot, o] = qid[q]


def build_hierarchy(leaves, dim: int, ns, num_ghost: int = 1, connect: str = "full"):
    """Level hierarchy from the finest leaves down to the single root patch.

    Returns a list of MeshLevel, finest first (P4estDomainGenerator::
    getFinestDomain / getCoarserDomain order)."""
    leaves = set(leaves)
    maxl = max(l for l, _ in leaves)
    ns = tuple(int(x) for x in ns)
    cur = sorted(leaves, key=lambda q: morton_key(dim, q, maxl))
    ids = {q: k for k, q in enumerate(cur)}
    levels = []
    curr_level = maxl
    prev = None  # (quads, lvl) of the finer level
    child_of = {}
    while True:
        P = len(cur)
        lvl = _empty_level(dim, P, ns, num_ghost)
        for k, q in enumerate(cur):
            l, c = q
            lvl.id[k] = ids[q]
            lvl.refine_level[k] = l
            lvl.child_ids[k, :] = child_of.get(q, [-1] * (1 << dim))
            h = 1.0 / (1 << l)
            for a in range(dim):
                st = c[a] * h
                up = (c[a] + 1) * h
                lvl.starts[k, a] = st
                lvl.spacings[k, a] = (up - st) / ns[a]
        lvl.quads = list(cur)
        _link_level(lvl, cur, connect)
        levels.append(lvl)
        if curr_level == 0:
            break
        # coarsen to curr_level - 1
        new_level = curr_level - 1
        nxt = []
        new_ids = {}
        child_of = {}
        fine = lvl
        seen = set()
        for k, q in enumerate(cur):
            l, c = q
            if q in seen:
                continue
            if l > new_level:
                parent = (l - 1, tuple(x >> 1 for x in c))
                fam = _children(dim, parent)
                sw_id = ids[fam[0]]
                seen.update(fam)
                child_of[parent] = [ids[ch] for ch in fam]
                new_ids[parent] = sw_id
                nxt.append(parent)
            else:
                child_of[q] = [ids[q]] + [-1] * ((1 << dim) - 1)
                new_ids[q] = ids[q]
                nxt.append(q)
        # parent links of the finer level
        for k, q in enumerate(cur):
            l, c = q
            if l > new_level:
                parent = (l - 1, tuple(x >> 1 for x in c))
                fine.parent_id[k] = new_ids[parent]
                fine.orth_on_parent[k] = sum((c[a] & 1) << a for a in range(dim))
            else:
                fine.parent_id[k] = ids[q]
                fine.orth_on_parent[k] = -1
        cur = sorted(nxt, key=lambda q: morton_key(dim, q, maxl))
        ids = new_ids
        curr_level = new_level
    return levels


# ---------------------------------------------------------------------------
# reference JSON mesh fixtures (json.cpp:160-300; test/utils/DomainReader.h)
# ---------------------------------------------------------------------------
_SIDE_NAMES = {2: ["WEST", "EAST", "SOUTH", "NORTH"],
               3: ["WEST", "EAST", "SOUTH", "NORTH", "BOTTOM", "TOP"]}
_CORNER_NAMES = {2: ["SW", "SE", "NW", "NE"],
                 3: ["BSW", "BSE", "BNW", "BNE", "TSW", "TSE", "TNW", "TNE"]}
_EDGE_NAMES = ["BS", "BN", "TS", "TN", "BW", "BE", "TW", "TE", "SW", "SE", "NW", "NE"]
_TYPE = {"NORMAL": NBR_NORMAL, "COARSE": NBR_COARSE, "FINE": NBR_FINE}


def _orth_from_json(val, m):
    if val is None:
        return -1
    if isinstance(val, int):
        return val
    names = {1: ["LOWER", "UPPER"], 2: ["SW", "SE", "NW", "NE"],
             3: ["BSW", "BSE", "BNW", "BNE", "TSW", "TSE", "TNW", "TNE"]}
    if val in ("NULL", "null"):
        return -1
    return names[m].index(val)


def _level_from_json(patches, dim, ns, num_ghost):
    P = len(patches)
    lvl = _empty_level(dim, P, ns, num_ghost)
    for k, pj in enumerate(patches):
        lvl.id[k] = pj["id"]
        lvl.refine_level[k] = pj.get("refine_level", -1)
        lvl.parent_id[k] = pj.get("parent_id", -1)
        lvl.orth_on_parent[k] = _orth_from_json(pj.get("orth_on_parent"), dim)
        if "child_ids" in pj:
            lvl.child_ids[k, :] = pj["child_ids"]
        for a in range(dim):
            lvl.starts[k, a] = pj["starts"][a]
            lvl.spacings[k, a] = pj["lengths"][a] / ns[a]
        for nb in pj.get("nbrs", []):
            s = _SIDE_NAMES[dim].index(nb["side"])
            slot = side_slot(dim, s)
            lvl.nbr_type[k, slot] = _TYPE[nb["type"]]
            for i, x in enumerate(nb["ids"]):
                lvl.nbr_ids[k, slot, i] = x
            if nb["type"] == "COARSE":
                lvl.nbr_orth[k, slot] = _orth_from_json(nb.get("orth_on_coarse"), dim - 1)
        for nb in pj.get("corner_nbrs", []):
            cidx = _CORNER_NAMES[dim].index(nb["corner"])
            slot = corner_slot(dim, cidx)
            lvl.nbr_type[k, slot] = _TYPE[nb["type"]]
            lvl.nbr_ids[k, slot, 0] = nb["ids"][0]
            if nb["type"] == "COARSE":
                lvl.nbr_orth[k, slot] = 0
        for nb in pj.get("edge_nbrs", []):
            e = _EDGE_NAMES.index(nb["edge"])
            slot = edge_slot(e)
            lvl.nbr_type[k, slot] = _TYPE[nb["type"]]
            for i, x in enumerate(nb["ids"]):
                lvl.nbr_ids[k, slot, i] = x
            if nb["type"] == "COARSE":
                lvl.nbr_orth[k, slot] = _orth_from_json(nb.get("orth_on_coarse"), 1)
    return lvl


def load_json_hierarchy(path, ns, num_ghost=1):
    with open(path) as fh:
        j = json.load(fh)
    dim = len(j["levels"][0][0]["starts"])
    return [_level_from_json(lv, dim, ns, num_ghost) for lv in j["levels"]]


_ORTH_NAMES = {1: ["LOWER", "UPPER"], 2: ["SW", "SE", "NW", "NE"],
               3: ["BSW", "BSE", "BNW", "BNE", "TSW", "TSE", "TNW", "TNE"]}
_TYPE_NAME = {NBR_NORMAL: "NORMAL", NBR_COARSE: "COARSE", NBR_FINE: "FINE"}


def _orth_to_json(v, m):
    # Orthant<0> and the null orthant are written as null (Orthant.cpp to_json)
    return None if m == 0 or v < 0 else _ORTH_NAMES[m][int(v)]


def _nbr_to_json(lvl, k, slot, m, key, name):
    """One neighbour entry (json.cpp to_json of Normal/Coarse/FineNbrInfo<m>): type, ids,
    ranks (one rank here), the coarse neighbour's orthant, and the face's name."""
    t = int(lvl.nbr_type[k, slot])
    n = (1 << m) if t == NBR_FINE else 1
    ids = [int(x) for x in lvl.nbr_ids[k, slot, :n]]
    nb = {"type": _TYPE_NAME[t], "ids": ids, "ranks": [0] * n}
    if t == NBR_COARSE:
        nb["orth_on_coarse"] = _orth_to_json(lvl.nbr_orth[k, slot], m)
    nb[key] = name
    return nb


def _level_to_json(lvl: MeshLevel):
    """The level's PatchInfos in the reference's JSON form (json.cpp:160-240), all on rank 0."""
    D = lvl.dim
    out = []
    for k in range(lvl.num_patches):
        pid = int(lvl.parent_id[k])
        pj = {"id": int(lvl.id[k]), "parent_id": pid, "parent_rank": 0 if pid >= 0 else -1,
              "orth_on_parent": _orth_to_json(lvl.orth_on_parent[k], D), "rank": 0,
              "starts": [float(x) for x in lvl.starts[k]],
              "lengths": [float(lvl.spacings[k, a] * lvl.ns[a]) for a in range(D)],
              "refine_level": int(lvl.refine_level[k])}
        pj["nbrs"] = [_nbr_to_json(lvl, k, side_slot(D, s), D - 1, "side", _SIDE_NAMES[D][s])
                      for s in range(2 * D) if lvl.nbr_type[k, side_slot(D, s)] != NBR_NONE]
        pj["edge_nbrs"] = [_nbr_to_json(lvl, k, edge_slot(e), 1, "edge", _EDGE_NAMES[e])
                           for e in range(12 if D == 3 else 0) if lvl.nbr_type[k, edge_slot(e)] != NBR_NONE]
        pj["corner_nbrs"] = [_nbr_to_json(lvl, k, corner_slot(D, c), 0, "corner", _CORNER_NAMES[D][c])
                             for c in range(1 << D) if lvl.nbr_type[k, corner_slot(D, c)] != NBR_NONE]
        # always written, -1 without children, as in test/mesh_inputs (json.cpp's to_json
        # omits them then; its from_json reads either)
        pj["child_ids"] = [int(x) for x in lvl.child_ids[k]]
        pj["child_ranks"] = [0 if x >= 0 else -1 for x in pj["child_ids"]]
        out.append(pj)
    return out


def save_json_hierarchy(levels, path):
    """Write a hierarchy (finest first) in the reference's mesh JSON format
    ({"levels": [[PatchInfo, ...], ...]}, as test/mesh_inputs), readable by
    load_json_hierarchy and by ThunderEgg's from_json (json.cpp:240-300)."""
    with open(path, "w") as fh:
        json.dump({"levels": [_level_to_json(lv) for lv in levels]}, fh)


def leaves_of_level(lvl: MeshLevel):
    """Recover (level, coords) of each patch from starts/spacings (unit cube)."""
    out = []
    for k in range(lvl.num_patches):
        length = lvl.spacings[k, 0] * lvl.ns[0]
        l = int(round(-math.log2(length)))
        c = tuple(int(round(lvl.starts[k, a] / length)) for a in range(lvl.dim))
        out.append((l, c))
    return out


# ---------------------------------------------------------------------------
# the workloads' meshes
# ---------------------------------------------------------------------------
def uniform_mesh(dim, level, n, num_ghost=1, connect="full"):
    return build_hierarchy(uniform_leaves(dim, level), dim, (n,) * dim, num_ghost, connect)


def circle_mesh(n=32, lo=3, hi=7, r=0.3, balance="full", num_ghost=1, connect="full"):
    leaves = circle_leaves(lo, hi, r)
    if balance:
        leaves = balance_leaves(leaves, 2, balance)
    return build_hierarchy(leaves, 2, (n, n), num_ghost, connect)


def random_mesh(seed, n=16, dim=2, lo=2, hi=6, p=0.3, num_ghost=1, connect="full"):
    leaves = balance_leaves(random_leaves(seed, dim, lo, hi, p), dim, "full")
    return build_hierarchy(leaves, dim, (n,) * dim, num_ghost, connect)


def cell_centers(lvl: MeshLevel):
    """Cell-centre coordinates of every interior cell, shape [P, *reversed(ns), D]
    (DomainTools::GetRealCoord, DomainTools.h:130-146)."""
    dim = lvl.dim
    grids = []
    for a in range(dim):
        i = np.arange(lvl.ns[a])
        grids.append(lvl.starts[:, a:a + 1] + lvl.spacings[:, a:a + 1] / 2.0
                     + lvl.spacings[:, a:a + 1] * i[None, :])
    P = lvl.num_patches
    shape = (P,) + tuple(lvl.ns[a] for a in reversed(range(dim)))
    out = np.empty(shape + (dim,))
    for a in range(dim):
        g = grids[a]
        sl = [slice(None)] + [None] * dim
        sl[dim - a] = slice(None)
        out[..., a] = np.broadcast_to(g[tuple(sl)], shape)
    return out


# ---------------------------------------------------------------------------
# batches: several independent hierarchies as one
# ---------------------------------------------------------------------------
def pad_hierarchy(levels, depth):
    """The hierarchy extended to `depth` levels by repeating its coarsest level: the patches
    of the old coarsest level are copied to each new level (parent = the patch itself, no
    orthant; the new level's patch has that one child), which is the reference's rule for
    patches that are not coarsened (P4estDomainGenerator.cpp:272-321).  A cycle on the
    padded hierarchy restricts into the copies and adds their corrections back; on a
    one-patch coarsest level, whose smooth is an exact solve, they change the result only by
    rounding.  Lets solves of different depths share one union hierarchy."""
    out = list(levels)
    if len(out) > depth:
        raise ValueError("the hierarchy is deeper than the requested depth")
    while len(out) < depth:
        c = out[-1]
        fine = dataclasses.replace(c, parent_id=c.id.copy(), orth_on_parent=np.full_like(c.orth_on_parent, -1))
        child = np.full_like(c.child_ids, -1)
        child[:, 0] = c.id
        coarse = dataclasses.replace(c, parent_id=np.full_like(c.parent_id, -1),
                                     orth_on_parent=np.full_like(c.orth_on_parent, -1), child_ids=child)
        out[-1] = fine
        out.append(coarse)
    return out


def union_hierarchy(hierarchies):
    """Concatenate the levels of several hierarchies of equal depth.

    Patches of solve b come after those of solve b-1 on every level, and every
    id is shifted by the sum of the previous solves' id ranges, so the union
    is a valid hierarchy of disconnected meshes.  Returns (levels, offsets)
    with offsets[k] the patch offsets of the solves on level k."""
    depth = len(hierarchies[0])
    if any(len(h) != depth for h in hierarchies):
        raise ValueError("hierarchies in one batch must have the same number of levels")
    shifts, acc = [], 0
    for h in hierarchies:
        shifts.append(acc)
        acc += int(max(int(lv.id.max()) for lv in h)) + 1
    if acc > np.iinfo(np.int32).max:
        raise ValueError("the union's patch ids exceed the int32 range")
    shifts = np.asarray(shifts, dtype=np.int32)

    levels, offsets = [], []
    for k in range(depth):
        parts = [h[k] for h in hierarchies]
        d0 = parts[0]
        for p in parts:
            if p.dim != d0.dim or tuple(p.ns) != tuple(d0.ns) or p.num_ghost != d0.num_ghost:
                raise ValueError("hierarchies in one batch must share patch shape")
        counts = np.array([p.num_patches for p in parts])
        s = np.repeat(shifts, counts)  # the id shift of every union patch

        def cat(name):
            return np.concatenate([getattr(p, name) for p in parts], axis=0)

        # every id moves by its solve's shift; absent links (-1, or a missing neighbour) stay
        parent, child = cat("parent_id"), cat("child_ids")
        nbr_type, nbr_ids = cat("nbr_type"), cat("nbr_ids")
        valid = (nbr_type >= 0)[:, :, None] & (nbr_ids >= 0)
        lv = MeshLevel(
            dim=d0.dim, ns=tuple(d0.ns), num_ghost=d0.num_ghost,
            id=(cat("id") + s).astype(np.int32), refine_level=cat("refine_level"),
            parent_id=np.where(parent >= 0, parent + s, parent).astype(np.int32),
            orth_on_parent=cat("orth_on_parent"),
            child_ids=np.where(child >= 0, child + s[:, None], child).astype(np.int32),
            starts=cat("starts"), spacings=cat("spacings"), nbr_type=nbr_type,
            nbr_ids=np.where(valid, nbr_ids + s[:, None, None], nbr_ids).astype(np.int32),
            nbr_orth=cat("nbr_orth"))
        assert lv.nbr_type.shape[1] == num_face_slots(d0.dim)
        levels.append(lv)
        offsets.append([0] + np.cumsum(counts).tolist())
    return levels, offsets
