"""Host logic of the Brownian-dynamics sampler (spme_gb300/bd.py) on the CPU: a
dense symmetric positive definite matrix stands in for the mobility operator
(the engine's `apply(f, u)` contract), and the block Lanczos M^{1/2} z is
checked against M^{1/2} from an eigendecomposition."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from spme_gb300 import bd  # noqa: E402


class DenseOperator:
    """u <- A f for each row of f (the engine's apply contract)."""

    def __init__(self, A):
        self.A = A
        self.applies = 0

    def apply(self, f, u):
        u.copy_(f @ self.A.T)
        self.applies += 1
        return u


def spd(n, cond, seed):
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    w = np.geomspace(1.0, cond, n)
    return (Q * w) @ Q.T


def sqrtm_apply(A, z):
    w, Q = np.linalg.eigh(A)
    return ((Q * np.sqrt(w)) @ Q.T @ z.T).T


@pytest.mark.parametrize("cond", [10.0, 1e3])
def test_lanczos_sqrt_matches_eigendecomposition(cond):
    n, R = 60, 3
    A = spd(n, cond, seed=int(cond))
    z = np.random.default_rng(7).standard_normal((R, n))
    op = DenseOperator(torch.tensor(A))
    y, iters = bd.sqrt_mobility_apply(op, torch.tensor(z), tol=1e-12, max_iter=n)
    ref = sqrtm_apply(A, z)
    err = np.linalg.norm(y.numpy() - ref) / np.linalg.norm(ref)
    assert err < 1e-8
    assert iters <= n and op.applies == iters  # one batched apply per iteration


def test_lanczos_stops_on_an_invariant_subspace():
    # z in a 2-dimensional eigenspace: exact after at most 2 iterations
    n = 40
    A = spd(n, 50.0, seed=3)
    w, Q = np.linalg.eigh(A)
    z = (Q[:, 5] + 2.0 * Q[:, 17])[None, :]
    y, iters = bd.sqrt_mobility_apply(DenseOperator(torch.tensor(A)), torch.tensor(z),
                                      tol=1e-14, max_iter=n)
    assert iters <= 3
    assert np.allclose(y.numpy(), sqrtm_apply(A, z), rtol=1e-10, atol=1e-12)


def test_brownian_displacements_drift_and_noise_scaling():
    n, R = 30, 2
    A = spd(n, 20.0, seed=5)
    F = np.random.default_rng(11).standard_normal((R, n))
    op = DenseOperator(torch.tensor(A))
    # kT = 0: the displacement is the drift s dt A F
    dx, _ = bd.brownian_displacements(op, torch.tensor(F), dt=0.01, kT=0.0,
                                      mobility_scale=0.5)
    assert np.allclose(dx.numpy(), 0.5 * 0.01 * F @ A.T, rtol=1e-12, atol=1e-14)
    # zero forces: the displacement is sqrt(2 kT dt s) M^{1/2} xi with the same xi the
    # generator gives
    g = torch.Generator().manual_seed(1234)
    dx, _ = bd.brownian_displacements(op, torch.zeros((R, n), dtype=torch.float64), dt=0.01,
                                      kT=2.0, mobility_scale=0.5, generator=g, tol=1e-12,
                                      max_iter=n)
    xi = torch.randn((R, n), generator=torch.Generator().manual_seed(1234),
                     dtype=torch.float64).numpy()
    ref = np.sqrt(2.0 * 2.0 * 0.01 * 0.5) * sqrtm_apply(A, xi)
    assert np.linalg.norm(dx.numpy() - ref) <= 1e-8 * np.linalg.norm(ref)
