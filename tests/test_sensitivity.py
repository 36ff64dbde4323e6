"""Host-side pieces of the sensitivity harness (no GPU)."""
import numpy as np
import pytest

from cassandra_gb300.autograd import fluctuation_sensitivity


def test_fluctuation_formula_on_a_gaussian_model():
    # U(x; theta) = theta x^2 / 2 at beta = 1: <x^2> = 1/theta, d<x^2>/dtheta = -1/theta^2
    rng = np.random.default_rng(0)
    theta = 2.0
    x = rng.normal(scale=theta ** -0.5, size=400_000)
    a = x * x
    d = fluctuation_sensitivity(a, 0.5 * x * x, beta=1.0)
    assert abs(d - (-1.0 / theta ** 2)) < 0.01


def test_lorentz_berthelot_tables():
    torch = pytest.importorskip("torch")
    from cassandra_gb300.autograd import _split_symmetric, lorentz_berthelot
    e, s = lorentz_berthelot(torch.tensor([1.0, 4.0], dtype=torch.float64), torch.tensor([3.0, 4.0], dtype=torch.float64))
    assert torch.allclose(e, torch.tensor([[1.0, 2.0], [2.0, 4.0]], dtype=torch.float64))
    assert torch.allclose(s, torch.tensor([[3.0, 3.5], [3.5, 4.0]], dtype=torch.float64))
    d = _split_symmetric(np.array([[1.0, 2.0], [2.0, 3.0]]))
    assert np.allclose(d, [[1.0, 1.0], [1.0, 3.0]])
