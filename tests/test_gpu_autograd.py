"""Test-only torch.autograd binding of the exact action gradient: the whole-ring action S(R) as a
differentiable torch function whose backward pass is the library's hand-written dS/dR, checked
by torch.autograd.gradcheck (central differences in float64) on small trapped-Coulomb and
electron-gas paths. The binding lives here, with the tests: the library itself has no torch
types in its interface."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from simpimc_gb300 import Simulation  # noqa: E402
from simpimc_gb300.configs import electron_gas, trapped_coulomb  # noqa: E402

pytestmark = pytest.mark.gpu


class PathAction(torch.autograd.Function):
    """S(R) of every action of `sim` at level 0 over the whole ring; backward = exact dS/dR."""

    @staticmethod
    def forward(ctx, R, sim):
        sim.set_path(R.detach().cpu().numpy().astype(np.float64), 2)
        ctx.sim = sim
        ctx.grad = torch.from_numpy(sim.action_gradient_path(-1, 0)).to(R.dtype)
        return torch.tensor(sim.total_action(-1, 0), dtype=R.dtype)

    @staticmethod
    def backward(ctx, g):
        return g * ctx.grad, None


@pytest.mark.parametrize("system", ["trap", "egas"])
def test_gradcheck(tmp_path, gpu_lib, system):
    if system == "trap":
        xml, path = trapped_coulomb(tmp_path, n_part=3, n_bead=4, n_level=1, seed=5)
    else:
        xml, path = electron_gas(tmp_path, n_part=4, n_bead=4, n_level=1, rs=1.5, k_cut_units=3.0, seed=7)
        L = (4 * np.pi * 4 / 3) ** (1 / 3) * 1.5
        path = np.random.default_rng(7).uniform(-L / 2, L / 2, size=path.shape)
    sim = Simulation(xml, base_dir=tmp_path)
    R = torch.tensor(path, dtype=torch.float64, requires_grad=True)
    assert torch.autograd.gradcheck(lambda x: PathAction.apply(x, sim), (R,), eps=1e-6, atol=1e-5, rtol=1e-5)
    sim.close()


def test_backward_drives_a_descent_step(tmp_path, gpu_lib):
    """One gradient-descent step through the binding lowers the action, as it must for a
    correct gradient."""
    xml, path = trapped_coulomb(tmp_path, n_part=4, n_bead=8, n_level=2, seed=21)
    sim = Simulation(xml, base_dir=tmp_path)
    R = torch.tensor(path, dtype=torch.float64, requires_grad=True)
    S0 = PathAction.apply(R, sim)
    S0.backward()
    with torch.no_grad():
        R2 = R - 1e-3 * R.grad
    S1 = PathAction.apply(R2, sim)
    assert float(S1.detach()) < float(S0.detach())
    sim.close()
