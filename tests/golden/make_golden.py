"""Write the golden fixtures of tests/golden/ from ThunderEgg itself.

Run in a tree where the reference sources exist (their recipe is
oracle/Makefile, target `ref`, which compiles them into oracle/_ref/libteref.so):

    python tests/golden/make_golden.py

Each fixture stores the flattened mesh levels (te_level_desc arrays) and the
reference's outputs for every operation on seeded inputs, so the oracle and
the GPU path can be checked against the reference where its sources are
absent.  The inputs are not stored: inputs() regenerates them from
numpy.random.default_rng(1234) in a fixed order.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from thunderegg_gb300 import mesh as M  # noqa: E402

LEVEL_FIELDS = ("id", "refine_level", "parent_id", "orth_on_parent", "child_ids", "starts", "spacings",
                "nbr_type", "nbr_ids", "nbr_orth")


def meshes():
    """Small meshes covering uniform, adaptive, odd-size and 3D cases."""
    return {
        "2d_uniform_n8": (M.uniform_mesh(2, 2, 8), (0, 1)),
        "2d_circle_n6": (M.circle_mesh(n=6, lo=2, hi=4), (0, 1)),
        "2d_random_n6": (M.random_mesh(3, n=6, lo=1, hi=3), (0, 1)),
        "2d_random_n5": (M.random_mesh(4, n=5, lo=1, hi=4), (1,)),
        "3d_uniform_n4": (M.uniform_mesh(3, 1, 4), (2,)),
        "3d_random_n4": (M.random_mesh(5, n=4, dim=3, lo=1, hi=2), (2,)),
    }


def pack_levels(levels, out, prefix="L"):
    out[f"{prefix}_count"] = np.array(len(levels))
    for k, lv in enumerate(levels):
        out[f"{prefix}{k}_meta"] = np.array([lv.dim, *lv.ns, lv.num_ghost])
        for f in LEVEL_FIELDS:
            out[f"{prefix}{k}_{f}"] = getattr(lv, f)


def unpack_levels(z, prefix="L"):
    levels = []
    for k in range(int(z[f"{prefix}_count"])):
        meta = z[f"{prefix}{k}_meta"]
        dim = int(meta[0])
        ns = tuple(int(x) for x in meta[1:1 + dim])
        lv = M._empty_level(dim, len(z[f"{prefix}{k}_id"]), ns, int(meta[-1]))
        for f in LEVEL_FIELDS:
            setattr(lv, f, np.array(z[f"{prefix}{k}_{f}"]))
        levels.append(lv)
    return levels


def inputs(levels, schemes):
    """The seeded inputs of every fixture entry, drawn in a fixed order."""
    rng = np.random.default_rng(1234)
    lv = levels[0]
    fts = (0, 2) if lv.dim == 2 else (0, 1, 2)
    inp = {}
    for sc in schemes:
        for ft in fts:
            inp[f"fill_s{sc}_f{ft}_in"] = rng.standard_normal(lv.padded_shape(2))
    inp["coeffs"] = 1 + 0.5 * rng.random(lv.padded_shape(1))
    for kind in (0, 1):
        inp[f"apply_k{kind}_in"] = rng.standard_normal(lv.padded_shape(1))
        inp[f"modrhs_k{kind}_f"] = rng.standard_normal(lv.padded_shape(1))
    inp["ps_f"] = rng.standard_normal(lv.padded_shape(1))
    inp["ps_u"] = rng.standard_normal(lv.padded_shape(1))
    if len(levels) > 1:
        inp["tr_fine"] = rng.standard_normal(lv.padded_shape(1))
        inp["tr_coarse"] = rng.standard_normal(levels[1].padded_shape(1))
        inp["gmg_f"] = rng.standard_normal(lv.padded_shape(1))
    return inp


def main():
    import oracle as orc

    orc.build(ref=True)
    R = orc.Oracle("teref")
    for name, (levels, schemes) in meshes().items():
        inp = inputs(levels, schemes)
        out = {}
        pack_levels(levels, out)
        lv = levels[0]
        fts = (0, 2) if lv.dim == 2 else (0, 1, 2)
        out["schemes"] = np.array(schemes)
        # ghost filling, every scheme and fill type, two components
        for sc in schemes:
            for ft in fts:
                out[f"fill_s{sc}_f{ft}_out"] = R.ghost_fill(lv, inp[f"fill_s{sc}_f{ft}_in"].copy(), sc, ft, 2)
                out[f"calls_f{ft}"] = R.ghost_calls(lv, ft)
        sc = schemes[0]
        coeffs = inp["coeffs"]
        for kind in (0, 1):
            uo, fo = R.apply(lv, inp[f"apply_k{kind}_in"].copy(), sc, 0, kind, 0, coeffs if kind else None)
            out[f"apply_k{kind}_u"] = uo
            out[f"apply_k{kind}_f"] = fo
            out[f"modrhs_k{kind}_out"] = R.modify_rhs(lv, uo, inp[f"modrhs_k{kind}_f"], sc, 0, kind,
                                                      coeffs if kind else None)
        for sm in (0, 1):
            for mode in (0, 1):
                out[f"ps_s{sm}_m{mode}"], _ = R.patch_solver(lv, inp["ps_f"], inp["ps_u"], sc, smoother=sm, mode=mode)
        if len(levels) > 1:
            for ex in (0, 1):
                out[f"restrict_e{ex}"] = R.restrict(levels[0], levels[1], inp["tr_fine"], ex)
            out["interp"] = R.interpolate(levels[1], levels[0], inp["tr_coarse"], inp["tr_fine"])
            cfg = orc.gmg_config(scheme=sc, smoother=0, tol=1e-10)
            out["vcycle"] = R.vcycle(levels, inp["gmg_f"], cfg)
            for ct in ("W", "F"):  # WCycle / FMGCycle through CycleBuilder's cycle_type
                cfg_t = orc.gmg_config(scheme=sc, smoother=0, tol=1e-10, cycle_type=ct)
                out[f"cycle_{ct}"] = R.vcycle(levels, inp["gmg_f"], cfg_t)
            us, its, res, rc = R.solve(levels, inp["gmg_f"], cfg)
            out["solve_u"], out["solve_its"] = us, np.array(its)
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **out)
        print(f"wrote {path} ({os.path.getsize(path) // 1024} KiB)")


if __name__ == "__main__":
    main()
