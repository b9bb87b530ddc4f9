"""OctreeSmokeFunction's host logic on the CPU with a stand-in solver: what it loads, how many steps
it runs with the tape on, which cotangent it seeds and which gradients it hands back to torch."""
import numpy as np
import pytest

import ast_solver

torch = pytest.importorskip("torch")


class FakeSolver:
    """Records the calls; the 'step' adds 0.5 * source density to the density and the 'backward'
    returns fixed multiples of the seeded cotangent."""

    def __init__(self, S):
        self.S = S
        self.calls = []
        self.arrays = {"density_oct": np.zeros(S)}

    def set_tensor(self, name, t):
        self.calls.append(("set", name, tuple(t.shape)))
        self.arrays[name] = t.detach().cpu().numpy().astype(np.float64).copy()

    def get_tensor(self, name, device="cpu"):
        self.calls.append(("get", name))
        a = self.arrays[name]
        return torch.tensor(a, dtype=torch.float64, device=device)

    def tape_start(self, every):
        self.calls.append(("tape", every))

    def update(self, dt):
        self.calls.append(("step", dt))
        self.arrays["density_oct"] = self.arrays["density_oct"] + 0.5 * self.arrays["source_density_oct"]

    def adjoint_reset(self):
        self.calls.append(("reset",))

    def backward(self):
        self.calls.append(("backward",))
        g = self.arrays["adj_density_oct"]
        S = self.S
        self.arrays["adj_mac"] = np.tile(2 * g, (3, 1))
        self.arrays["adj_tilt_vel"] = np.tile(3 * g[:, None], (1, 8))
        self.arrays["adj_source_density_oct"] = 4 * g
        self.arrays["adj_source_density_tilt"] = np.zeros(S)
        return "stats"


def test_forward_and_backward_plumbing():
    S = 5
    s = FakeSolver(S)
    mac = torch.zeros(3, S, dtype=torch.float64, requires_grad=True)
    tilt = torch.zeros(S, 8, dtype=torch.float64, requires_grad=True)
    src_o = torch.full((S,), 2.0, dtype=torch.float64, requires_grad=True)
    src_t = torch.ones(S, dtype=torch.float64, requires_grad=True)
    out = ast_solver.OctreeSmokeFunction.apply(s, 3, 0.01, 16, mac, tilt, src_o, src_t)
    assert torch.allclose(out, torch.full((S,), 3.0, dtype=torch.float64))  # 3 steps of 0.5 * 2
    names = [c[1] for c in s.calls if c[0] == "set"]
    assert names == ["mac", "tilt_vel", "source_density_oct", "source_density_tilt"]
    kinds = [c[0] for c in s.calls]
    assert kinds.index("tape") < kinds.index("step")
    assert ("tape", 16) in s.calls and kinds.count("step") == 3
    w = torch.arange(S, dtype=torch.float64)
    (out * w).sum().backward()
    assert ("reset",) in s.calls and ("backward",) in s.calls
    assert s.calls.index(("reset",)) < s.calls.index(("backward",))
    assert np.allclose(s.arrays["adj_density_oct"], w.numpy())
    assert torch.allclose(mac.grad, 2 * w.expand(3, S))
    assert torch.allclose(tilt.grad, 3 * w[:, None].expand(S, 8))
    assert torch.allclose(src_o.grad, 4 * w)
    assert torch.allclose(src_t.grad, torch.zeros(S, dtype=torch.float64))


def test_adjoint_names_have_state_shapes():
    assert ast_solver._base("adj_mac") == "mac"
    assert ast_solver._dtype("adj_tilt_vel") is np.float64
    assert ast_solver._dtype("source_density_oct") is np.float64
    assert ast_solver._dtype("adj_source_density_tilt") is np.float64
