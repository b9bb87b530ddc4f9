"""Reverse mode of the octree smoke step (astg_adjoint.cu) through the C ABI.

* The samplers' weight enumeration reproduces the forward samplers (value) and the central
  difference of the forward sampler (position gradient).
* Dot-product tests: for each stage and for the whole step, <J d, y> from central differences of
  the forward equals <d, J^T y> from the transposes, for random d and y over the whole state.
* The gradient of a 32-step window (32^3 coarsest cells, 2 levels, topology frozen after 4 adaptive
  steps) of L = ||density - g||_2 with respect to the initial face velocities and the per-slot
  source densities matches central differences (eps 1e-6) along 20 seeded unit directions to 1e-4,
  with the pressure solves run to a relative residual of 1e-13 so that the finite differences
  resolve the derivative.
* The checkpointed tape (recompute) gives the gradient of the stored tape; the torch
  autograd.Function returns the same gradients.
"""
import numpy as np
import pytest

import ast_solver

pytestmark = pytest.mark.gpu

STATE = ["density_oct", "density_tilt", "heat_oct", "heat_tilt", "mac", "tilt_vel", "dual_oct", "dual_tilt"]
DT = 0.01


def frozen(coarsest=8, levels=3, warm=4, frozen_steps=2, tol=1e-13):
    """A handle whose tilts opened during `warm` adaptive steps, then frozen."""
    s = ast_solver.OctreeSmoke3(coarsest, levels)
    for _ in range(warm):
        s.update(DT)
    s.set_tilt_adaptivity(False)
    s.set_solver_parameters(tol, 3000)
    for _ in range(frozen_steps):
        s.update(DT)
    return s


def get_state(s, prefix=""):
    return {k: s.get(prefix + k).copy() for k in STATE}


def set_state(s, st, prefix=""):
    for k, v in st.items():
        s.set(prefix + k, v)


def vdot(a, b):
    return sum(float(np.vdot(a[k], b[k])) for k in a)


def run_map(s, stage, X, Pt):
    set_state(s, X)
    set_state(s, Pt, "t_")
    if stage == "step":
        s.update(DT)
    else:
        s.stage(stage, DT)
    return get_state(s)


def wall_normal_faces(s):
    """(3, S) mask of the MAC faces the closed walls zero (x-, x+, y-, y+, z-)."""
    coords, sizes = s.get("slot_coords"), s.get("level_sizes")
    lev = np.repeat(np.arange(len(sizes)), sizes[:, 2])
    r = s.size(2) >> lev
    x, y, z = coords[:, 0], coords[:, 1], coords[:, 2]
    return np.stack([(x == 0) | (x == r - 1), (y == 0) | (y == r - 1), z == 0])


def dot_test(s, stage, eps, seed):
    rng = np.random.default_rng(seed)
    X, Pt = get_state(s), get_state(s, "t_")
    d = {k: rng.standard_normal(v.shape) * max(1e-3, float(np.abs(v).max())) for k, v in X.items()}
    if stage == 5:
        # a wall-normal face traces back along the wall, where the interpolation is clamped on one
        # side: its derivative is one-sided (the transpose takes the inner side) and a central
        # difference straddling the wall averages the two.  The step's wall stage zeroes these
        # faces before every advection, so the isolated stage is tested without moving them.
        d["mac"][wall_normal_faces(s)] = 0
    y = {k: rng.standard_normal(v.shape) for k, v in X.items()}
    Yp = run_map(s, stage, {k: X[k] + eps * d[k] for k in X}, Pt)
    Ym = run_map(s, stage, {k: X[k] - eps * d[k] for k in X}, Pt)
    jvp = vdot({k: (Yp[k] - Ym[k]) / (2 * eps) for k in X}, y)
    set_state(s, X)
    set_state(s, Pt, "t_")
    s.adjoint_reset()
    set_state(s, y, "adj_")
    if stage == "step":
        s.step_vjp(DT)
    else:
        s.stage_vjp(stage, DT)
    vjp = vdot(get_state(s, "adj_"), d)
    set_state(s, X)
    set_state(s, Pt, "t_")
    return jvp, vjp


@pytest.fixture(scope="module")
def small():
    s = frozen()
    yield s
    s.close()


def test_frozen_scene_has_open_tilts(small):
    opened = small.get("tilt_open") & 1
    assert opened.sum() > 0
    assert small.size(4) > 0  # half tilts


def test_probe_scalar_weights(small):
    rng = np.random.default_rng(1)
    pos = rng.uniform(0.03, 0.97, (4000, 3))
    pos[:2000] = 0.5 + (pos[:2000] - 0.5) * 0.3  # dense near the refined source region
    out = small.adjoint_probe(0, pos)
    assert np.allclose(out[:, 1], out[:, 0], rtol=1e-12, atol=1e-14)
    h = 1e-7
    ok = []
    for k in range(3):
        pp, pm = pos.copy(), pos.copy()
        pp[:, k] += h
        pm[:, k] -= h
        fd = (small.adjoint_probe(0, pp)[:, 0] - small.adjoint_probe(0, pm)[:, 0]) / (2 * h)
        scale = np.abs(out[:, 2 + k]).max() + 1e-12
        ok.append(np.abs(fd - out[:, 2 + k]) <= 1e-5 * scale + 1e-6 * np.abs(fd))
    ok = np.all(ok, axis=0)
    # points within h of a kink (cell faces, level boundaries, the tilt correction's min) differ
    assert ok.mean() > 0.99, ok.mean()


def test_probe_velocity_weights(small):
    rng = np.random.default_rng(2)
    pos = rng.uniform(0.03, 0.97, (4000, 3))
    pos[:2000] = 0.5 + (pos[:2000] - 0.5) * 0.3
    out = small.adjoint_probe(1, pos)
    assert np.allclose(out[:, 3:6], out[:, 0:3], rtol=1e-12, atol=1e-14)
    h = 1e-7
    ok = np.ones(len(pos), bool)
    J = out[:, 6:15].reshape(-1, 3, 3)
    for k in range(3):
        pp, pm = pos.copy(), pos.copy()
        pp[:, k] += h
        pm[:, k] -= h
        fd = (small.adjoint_probe(1, pp)[:, 0:3] - small.adjoint_probe(1, pm)[:, 0:3]) / (2 * h)
        scale = np.abs(J[:, :, k]).max() + 1e-12
        ok &= np.all(np.abs(fd - J[:, :, k]) <= 1e-5 * scale + 1e-6 * np.abs(fd), axis=1)
    assert ok.mean() > 0.99, ok.mean()


# linear stages are checked to rounding; the projection to its solver tolerance; advection and the
# whole step (nonlinear through the back-traced positions) with a small step
@pytest.mark.parametrize("stage,eps,rtol", [(0, 1e-2, 1e-9), (1, 1e-2, 1e-9), (2, 1e-2, 1e-9), (3, 1e-2, 1e-7),
                                            (4, 1e-2, 1e-9), (5, 1e-7, 1e-5), ("step", 1e-7, 1e-5)])
def test_vjp_dot_product(small, stage, eps, rtol):
    for seed in (3, 4):
        jvp, vjp = dot_test(small, stage, eps, seed)
        assert abs(jvp - vjp) <= rtol * max(abs(jvp), abs(vjp), 1e-30), (stage, jvp, vjp)


def cell_geometry(s):
    """Centres and volumes of the non-ghost octagon cells, and the mask of those slots."""
    coords = s.get("slot_coords")
    sizes = s.get("level_sizes")
    L = len(sizes)
    res0 = s.size(2)
    lev = np.repeat(np.arange(L), sizes[:, 2])
    h = (1.0 / res0) * (2.0 ** lev)
    ghost = (coords[:, 3] & 2) != 0
    res_l = (res0 >> lev)
    inner = np.all(coords[:, :3] < (res_l - 1)[:, None], axis=1)
    cells = ~ghost & inner
    centre = (coords[:, :3] + 0.5) * h[:, None]
    return centre, h ** 3, cells


class Window:
    """L = ||density - g||_2 after `steps` frozen steps as a function of (mac, tilt_vel, source
    densities) at the start; the starting state (both buffers) is restored before every run."""

    def __init__(self, s, steps):
        self.s, self.steps = s, steps
        self.X, self.Pt = get_state(s), get_state(s, "t_")
        centre, vol, cells = cell_geometry(s)
        r2 = ((centre - np.array([0.5, 0.5, 0.6])) ** 2).sum(1)
        self.g = np.exp(-r2 / (2 * 0.1 ** 2))
        self.w = np.where(cells, vol, 0.0)
        S = s.slots
        self.src0 = (np.ones(S), np.ones(S))

    def params(self):
        return [self.X["mac"].copy(), self.X["tilt_vel"].copy(), self.src0[0].copy(), self.src0[1].copy()]

    def loss(self, p, tape=None):
        s = self.s
        set_state(s, self.X)
        set_state(s, self.Pt, "t_")
        s.set("mac", p[0])
        s.set("tilt_vel", p[1])
        s.set("source_density_oct", p[2])
        s.set("source_density_tilt", p[3])
        if tape is not None:
            s.tape_start(tape)
        for _ in range(self.steps):
            s.update(DT)
        dens = s.get("density_oct")
        r = dens - self.g
        val = float(np.sqrt((self.w * r * r).sum()))
        return val, self.w * r / val

    def gradient(self, p, tape=0):
        val, seed = self.loss(p, tape)
        s = self.s
        s.adjoint_reset()
        s.set("adj_density_oct", seed)
        stats = s.backward()
        g = [s.get("adj_mac"), s.get("adj_tilt_vel"), s.get("adj_source_density_oct"),
             s.get("adj_source_density_tilt")]
        s.tape_stop()
        return val, g, stats


@pytest.fixture(scope="module")
def window():
    s = frozen(32, 2, warm=4, frozen_steps=1)
    w = Window(s, 32)
    yield w
    s.close()


def test_window_gradient_matches_finite_differences(window):
    p = window.params()
    val, g, stats = window.gradient(p, tape=0)
    assert stats.steps == 32 and stats.solves == 32 and stats.recomputed_steps == 0
    assert all(np.all(np.isfinite(x)) for x in g)
    rng = np.random.default_rng(20)
    eps = 1e-6
    errs = []
    for _ in range(20):
        d = [rng.standard_normal(x.shape) for x in p]
        nrm = np.sqrt(sum((x * x).sum() for x in d))
        d = [x / nrm for x in d]
        lp, _ = window.loss([a + eps * b for a, b in zip(p, d)])
        lm, _ = window.loss([a - eps * b for a, b in zip(p, d)])
        fd = (lp - lm) / (2 * eps)
        ad = sum(float(np.vdot(a, b)) for a, b in zip(g, d))
        errs.append(abs(fd - ad) / max(abs(fd), abs(ad), 1e-30))
    assert max(errs) <= 1e-4, errs


def test_checkpointed_tape_matches_stored_tape(window):
    p = window.params()
    v0, g0, s0 = window.gradient(p, tape=0)
    v1, g1, s1 = window.gradient(p, tape=8)
    assert v0 == v1
    assert s1.checkpoints == 4 and s1.recomputed_steps == 32
    for a, b in zip(g0, g1):
        assert np.allclose(a, b, rtol=1e-9, atol=1e-12 * np.abs(a).max())


def test_autograd_function(window):
    torch = pytest.importorskip("torch")
    s = window.s
    p = [torch.tensor(x, device="cuda", requires_grad=True) for x in window.params()]
    set_state(s, window.X)
    set_state(s, window.Pt, "t_")
    dens = ast_solver.OctreeSmokeFunction.apply(s, window.steps, DT, 0, *p)
    g = torch.tensor(window.g, device="cuda")
    w = torch.tensor(window.w, device="cuda")
    loss = torch.sqrt((w * (dens - g) ** 2).sum())
    loss.backward()
    v, ref, _ = window.gradient(window.params(), tape=0)
    assert abs(loss.item() - v) <= 1e-12 * v
    for t, r in zip(p, ref):
        assert np.allclose(t.grad.cpu().numpy(), r, rtol=1e-9, atol=1e-12 * np.abs(r).max())
    s.tape_stop()


def test_tape_refusals():
    s = ast_solver.OctreeSmoke3(8, 2)
    with pytest.raises(ast_solver.AstgError) as e:
        s.tape_start(0)  # tilt adaptivity is on: the topology is not frozen
    assert e.value.status == ast_solver.ASTG_BAD_ARG
    s.set_tilt_adaptivity(False)
    with pytest.raises(ast_solver.AstgError):
        s.backward()  # nothing taped
    s.tape_start(0)
    s.update(DT)
    with pytest.raises(ast_solver.AstgError):
        s.stage(1, DT)  # single stages would not be recorded
    with pytest.raises(ast_solver.AstgError):
        s.set_tilt_adaptivity(True)
    s.adjoint_reset()
    s.set("adj_density_oct", np.ones(s.slots))
    st = s.backward()
    assert st.steps == 1 and st.solves == 1
    s.tape_stop()
    s.stage(1, DT)  # allowed again
    s.close()
