"""Shared helpers: golden fixtures and array comparison."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
# state arrays of one buffer, in fixture/oracle naming
FIELDS = ["density_oct", "density_tilt", "heat_oct", "heat_tilt", "mac", "tilt_vel", "dual_oct", "dual_tilt",
          "tilt_e", "tilt_flags"]
LAYOUT = ["level_sizes", "slot_coords", "split_map", "half_tilts", "t_joints", "closed_by_half_tilt", "w_mac",
          "w_tilt"]
STAGES = ["scene", "force", "preproject", "project", "dual", "advect"]
PROJ = ["pindex_oct", "pindex_tilt", "A_rowptr", "A_col", "A_val", "b", "p", "pcg_iters"]

_cache = {}


def golden(name):
    if name not in _cache:
        with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
            _cache[name] = {k: z[k] for k in z.files}
    return _cache[name]


def case(name):
    c, lv, steps = golden(name)["meta/case"].tolist()
    return c, lv, steps


def state(g, prefix):
    """All arrays stored under prefix (e.g. 'step2/') with the prefix stripped."""
    return {k[len(prefix):]: v for k, v in g.items() if k.startswith(prefix)}


def max_rel(ref, got):
    ref = np.asarray(ref, dtype=np.float64).ravel()
    got = np.asarray(got, dtype=np.float64).ravel()
    both = np.isnan(ref) & np.isnan(got)
    d = np.abs(ref - got)
    d[both] = 0
    scale = np.abs(ref[~np.isnan(ref)]).max() if (~np.isnan(ref)).any() else 1.0
    return float(d.max() / max(scale, 1e-300)) if d.size else 0.0


def assert_same(name, ref, got, rel=0.0):
    ref = np.asarray(ref)
    got = np.asarray(got)
    assert ref.shape == got.shape, f"{name}: shape {ref.shape} != {got.shape}"
    if ref.dtype.kind in "iu" or rel == 0.0:
        if ref.dtype.kind == "f":
            same = (ref == got) | (np.isnan(ref) & np.isnan(got))
        else:
            same = ref == got
        bad = np.nonzero(~same.ravel())[0]
        assert bad.size == 0, (f"{name}: {bad.size} of {ref.size} differ, first at {bad[:4]}: "
                               f"ref {ref.ravel()[bad[:4]]} got {got.ravel()[bad[:4]]}")
    else:
        r = max_rel(ref, got)
        assert r <= rel, f"{name}: max relative difference {r:.3e} > {rel:.1e}"
