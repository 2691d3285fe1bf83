"""Mesh hierarchy builder: structure of the level tables (no GPU).

The reference builds its hierarchy with p4est (P4estDomainGenerator.cpp);
thunderegg_gb300.mesh re-creates the same semantics.  Checked here: the
neighbour relation is consistent in both directions, meshes are 2:1 balanced,
parent/child links follow the coarsening rule, and the benchmark meshes have
the level sizes of their specification.  Where the reference's own mesh
fixtures (test/mesh_inputs/*.json) exist, the builder reproduces them up to
the numbering of the patches.
"""
import glob
import json
import os

import numpy as np
import pytest

from thunderegg_gb300 import mesh as M

import oracle as _orc  # noqa: E402  (only for the location of the reference tree)

REF_MESHES = _orc.REF_MESH_INPUTS


def check_symmetric(lv):
    """Every Normal/Coarse/Fine side link has its inverse on the neighbour."""
    D = lv.dim
    idx = lv.id_to_local()
    for p in range(lv.num_patches):
        for side in range(2 * D):
            slot = M.side_slot(D, side)
            t = lv.nbr_type[p, slot]
            if t < 0:
                continue
            opp = M.side_slot(D, side ^ 1)
            if t == M.NBR_NORMAL:
                q = idx[lv.nbr_ids[p, slot, 0]]
                assert lv.nbr_type[q, opp] == M.NBR_NORMAL and lv.nbr_ids[q, opp, 0] == lv.id[p]
            elif t == M.NBR_COARSE:
                q = idx[lv.nbr_ids[p, slot, 0]]
                assert lv.nbr_type[q, opp] == M.NBR_FINE
                assert lv.nbr_ids[q, opp, lv.nbr_orth[p, slot]] == lv.id[p]
            else:
                for o in range(1 << (D - 1)):
                    q = idx[lv.nbr_ids[p, slot, o]]
                    assert lv.nbr_type[q, opp] == M.NBR_COARSE and lv.nbr_orth[q, opp] == o


@pytest.mark.parametrize("make", [lambda: M.uniform_mesh(2, 2, 8), lambda: M.circle_mesh(n=4),
                                  lambda: M.random_mesh(7, n=4), lambda: M.random_mesh(3, n=4, dim=3, lo=1, hi=3)])
def test_hierarchy_structure(make):
    levels = make()
    assert levels[-1].num_patches == 1
    for lv in levels:
        check_symmetric(lv)
        assert len(set(lv.id.tolist())) == lv.num_patches
    for fine, coarse in zip(levels[:-1], levels[1:]):
        cid = coarse.id_to_local()
        for p in range(fine.num_patches):
            assert fine.parent_id[p] in cid  # every fine patch has a parent on the next level
            c = cid[fine.parent_id[p]]
            if fine.orth_on_parent[p] >= 0:  # coarsened: the parent lists it at its orthant
                assert coarse.child_ids[c, fine.orth_on_parent[p]] == fine.id[p]
                assert coarse.refine_level[c] == fine.refine_level[p] - 1
            else:  # copied patch keeps its id
                assert fine.parent_id[p] == fine.id[p]


def test_benchmark_mesh_sizes():
    levels = M.circle_mesh(n=32)
    assert [lv.num_patches for lv in levels] == [1444, 976, 496, 220, 64, 16, 4, 1]
    assert [lv.num_patches for lv in M.uniform_mesh(2, 2, 32)] == [16, 4, 1]


def test_balance_is_two_to_one():
    leaves = M.balance_leaves(M.random_leaves(5, 2, 2, 6, 0.3), 2, "full")
    idx = M._LeafIndex(leaves, 2)
    for (l, c) in leaves:
        for d in [(-1, 0), (1, 0), (0, -1), (0, 1), (1, 1), (-1, -1), (1, -1), (-1, 1)]:
            q = idx.covering(l, (c[0] + d[0], c[1] + d[1]))
            assert q is None or q[0] >= l - 1


@pytest.mark.skipif(not os.path.isdir(REF_MESHES), reason="reference mesh fixtures not present")
@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(REF_MESHES, "*mpi1.json"))))
def test_builder_reproduces_reference_meshes(path):
    if "1x2" in path:
        pytest.skip("two-tree domain")
    j = json.load(open(path))
    dim = len(j["levels"][0][0]["starts"])
    ns = (4,) * dim
    ref = M.load_json_hierarchy(path, ns)
    mine = M.build_hierarchy(M.leaves_of_level(ref[0]), dim, ns)
    assert len(mine) == len(ref)

    def key(lv, k):
        return (round(lv.spacings[k, 0] * lv.ns[0], 12),) + tuple(round(x, 12) for x in lv.starts[k])

    maps = []
    for a, b in zip(ref, mine):
        bk = {key(b, i): i for i in range(b.num_patches)}
        maps.append(({int(a.id[i]): int(b.id[bk[key(a, i)]]) for i in range(a.num_patches)}, bk))
    for k, (a, b) in enumerate(zip(ref, mine)):
        m, bk = maps[k]
        for i in range(a.num_patches):
            j2 = bk[key(a, i)]
            if k + 1 < len(ref):
                assert maps[k + 1][0][int(a.parent_id[i])] == b.parent_id[j2]
                assert a.orth_on_parent[i] == b.orth_on_parent[j2]
            for s in range(M.num_face_slots(dim)):
                assert a.nbr_type[i, s] == b.nbr_type[j2, s]
                t = a.nbr_type[i, s]
                if t < 0:
                    continue
                nn = 1
                if t == M.NBR_FINE:
                    nn = (1 << (dim - 1)) if s >= (4 if dim == 2 else 20) else (2 if (dim == 3 and s >= 8) else 1)
                assert [m[int(x)] for x in a.nbr_ids[i, s, :nn]] == list(b.nbr_ids[j2, s, :nn])
                if t == M.NBR_COARSE:
                    assert a.nbr_orth[i, s] == b.nbr_orth[j2, s]


def test_union_hierarchy_shifts_each_solve():
    """Every level of a union lists each solve's patches in order, every id of solve b
    shifted by the id ranges of the solves before it, and absent links left at -1."""
    hs = [M.circle_mesh(n=8, lo=2, hi=4), M.uniform_mesh(2, 2, 8), M.circle_mesh(n=8, lo=2, hi=4)]
    hs = [h[:3] for h in hs]
    union, offs = M.union_hierarchy(hs)
    shift = np.cumsum([0] + [max(int(lv.id.max()) for lv in h) + 1 for h in hs])[:-1]
    for k, lv in enumerate(union):
        assert offs[k][-1] == lv.num_patches
        for b, h in enumerate(hs):
            part, sl, s = h[k], slice(offs[k][b], offs[k][b + 1]), int(shift[b])
            assert np.array_equal(lv.id[sl], part.id + s)
            assert np.array_equal(lv.parent_id[sl], np.where(part.parent_id >= 0, part.parent_id + s, -1))
            assert np.array_equal(lv.child_ids[sl], np.where(part.child_ids >= 0, part.child_ids + s, -1))
            has = (part.nbr_type >= 0)[:, :, None] & (part.nbr_ids >= 0)
            assert np.array_equal(lv.nbr_ids[sl], np.where(has, part.nbr_ids + s, part.nbr_ids))
            for name in ("refine_level", "orth_on_parent", "starts", "spacings", "nbr_type", "nbr_orth"):
                assert np.array_equal(getattr(lv, name)[sl], getattr(part, name))
        assert lv.id.dtype == np.int32 and lv.nbr_ids.dtype == np.int32
        # ids stay unique across the solves
        assert len(np.unique(lv.id)) == lv.num_patches


def _same_tables(a, b, exact_geometry=True):
    for la, lb in zip(a, b):
        for f in ("id", "refine_level", "parent_id", "orth_on_parent", "child_ids", "nbr_type", "nbr_ids",
                  "nbr_orth"):
            assert np.array_equal(getattr(la, f), getattr(lb, f)), f
        for f in ("starts", "spacings"):
            x, y = getattr(la, f), getattr(lb, f)
            assert np.array_equal(x, y) if exact_geometry else np.allclose(x, y, rtol=1e-15, atol=0), f


@pytest.mark.skipif(not os.path.isdir(REF_MESHES), reason="reference mesh fixtures not present")
@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(REF_MESHES, "*.json"))))
def test_json_round_trip_of_reference_meshes(path, tmp_path):
    """The reference's mesh inputs read, written back in the same format and read again
    give the same tables (ranks are not kept: everything is rank 0 here)."""
    j = json.load(open(path))
    dim = len(j["levels"][0][0]["starts"])
    ns = (4,) * dim
    ref = M.load_json_hierarchy(path, ns)
    out = tmp_path / "mesh.json"
    M.save_json_hierarchy(ref, out)
    _same_tables(ref, M.load_json_hierarchy(out, ns))
    # the written patches carry the reference's keys
    w = json.load(open(out))["levels"][0][0]
    assert set(j["levels"][0][0]) <= set(w) | {"forest"}


@pytest.mark.parametrize("make", [lambda: M.circle_mesh(n=8, lo=2, hi=5), lambda: M.random_mesh(11, n=4, dim=3, lo=1, hi=3),
                                  lambda: M.uniform_mesh(3, 2, 8)])
def test_json_round_trip_of_built_meshes(make, tmp_path):
    levels = make()
    out = tmp_path / "mesh.json"
    M.save_json_hierarchy(levels, out)
    _same_tables(levels, M.load_json_hierarchy(out, levels[0].ns))


@pytest.mark.parametrize("make", [lambda: M.circle_mesh(n=8, lo=2, hi=5), lambda: M.random_mesh(11, n=4, dim=3, lo=1, hi=3)])
def test_reference_reads_written_json(make, tmp_path):
    """ThunderEgg's own from_json (compiled from the reference sources) reads every level of
    a file written by save_json_hierarchy into a Domain whose tables are this builder's."""
    import ctypes

    import oracle as orc

    if not orc.ref_sources_present():
        pytest.skip("reference sources not present")

    orc.build(ref=True)
    lib = ctypes.CDLL(orc.REF_LIB)
    levels = make()
    out = tmp_path / "mesh.json"
    M.save_json_hierarchy(levels, out)
    text = json.load(open(out))["levels"]
    for lv, lj in zip(levels, text):
        outs = {}
        args = []
        for name in ("id", "refine_level", "parent_id", "orth_on_parent", "child_ids", "starts", "spacings",
                     "nbr_type", "nbr_ids", "nbr_orth"):
            want = np.asarray(getattr(lv, name))
            a = np.zeros(want.shape, dtype=np.float64 if want.dtype == np.float64 else np.int32)
            outs[name] = a
            ct = ctypes.c_double if a.dtype == np.float64 else ctypes.c_int
            args.append(a.ctypes.data_as(ctypes.POINTER(ct)))
        rc = lib.teref_json_level(json.dumps(lj).encode(), lv.dim, lv.ns[0], lv.num_ghost, lv.num_patches, *args)
        assert rc == 0
        # a coarse corner neighbour's Orthant<0> is written as null (Orthant.cpp to_json) and read
        # back as the null orthant (index 1); Orthant<0> has one orthant, so both name the same
        # neighbour (the reference's own write-then-read changes it the same way)
        corner = np.zeros(lv.nbr_orth.shape, dtype=bool)
        corner[:, [M.corner_slot(lv.dim, c) for c in range(1 << lv.dim)]] = True
        coarse_corner = corner & (lv.nbr_type == M.NBR_COARSE)
        assert np.isin(outs["nbr_orth"][coarse_corner], (0, 1)).all()
        outs["nbr_orth"][coarse_corner] = lv.nbr_orth[coarse_corner]
        for name, a in outs.items():
            assert np.array_equal(a, np.asarray(getattr(lv, name))), name


def test_pad_hierarchy_copies_the_coarsest_level():
    """pad_hierarchy extends a hierarchy with copied levels: the old coarsest patches point to
    themselves with a null orthant, each copy has that patch as its only child; a padded
    hierarchy joins a deeper one in a union."""
    shallow, deep = M.uniform_mesh(2, 1, 8), M.circle_mesh(n=8, lo=2, hi=4)
    padded = M.pad_hierarchy(shallow, len(deep))
    assert len(padded) == len(deep)
    for k in range(len(shallow) - 1):
        assert np.array_equal(padded[k].parent_id, shallow[k].parent_id)
    for k in range(len(shallow) - 1, len(deep)):
        lv = padded[k]
        assert np.array_equal(lv.id, shallow[-1].id) and np.array_equal(lv.nbr_type, shallow[-1].nbr_type)
        if k + 1 < len(deep):
            assert np.array_equal(lv.parent_id, lv.id) and np.all(lv.orth_on_parent == -1)
        else:
            assert np.all(lv.parent_id == -1)
        if k >= len(shallow):
            assert np.array_equal(lv.child_ids[:, 0], lv.id) and np.all(lv.child_ids[:, 1:] == -1)
    levels, offsets = M.union_hierarchy([padded, deep])
    assert [lv.num_patches for lv in levels] == [a.num_patches + b.num_patches for a, b in zip(padded, deep)]
    with pytest.raises(ValueError):
        M.pad_hierarchy(deep, 2)
