"""Brownian-dynamics displacements with the SPME-RPY mobility.

A Brownian step needs the deterministic drift M F and a random displacement
with covariance 2 kT dt M, i.e. M^{1/2} z for Gaussian z.  M is only
available as an operator, so M^{1/2} z comes from the Lanczos process
(Chow & Saad, SIAM J. Sci. Comput. 36 (2014) A237): after m steps
    M^{1/2} z ~= |z| V_m T_m^{1/2} e_1,
V_m the Lanczos basis and T_m the tridiagonal projection.  The R vectors
z_1..z_R run their Lanczos recurrences in lockstep, so each iteration is one
apply of M to a block of R right-hand sides — the batched mesh pass of the
engine.  All vector algebra stays on the device (torch); the m x m
eigenproblems are tiny.
"""
from __future__ import annotations

import torch


def _sqrt_tridiag_e1(alpha, beta):
    """T^{1/2} e_1 for symmetric tridiagonal T (batch of R): alpha (R, m),
    beta (R, m-1).  Negative Ritz values (round-off) are clipped to zero."""
    R, m = alpha.shape
    T = torch.diag_embed(alpha)
    if m > 1:
        T = T + torch.diag_embed(beta, offset=1) + torch.diag_embed(beta, offset=-1)
    w, Q = torch.linalg.eigh(T.double())
    s = torch.sqrt(torch.clamp(w, min=0.0))
    return (Q * s.unsqueeze(1)) @ Q[:, 0, :].unsqueeze(-1)  # (R, m, 1)


def sqrt_mobility_apply(engine, z, tol: float = 1e-4, max_iter: int = 60,
                        reorthogonalize: bool = True):
    """y ~= M^{1/2} z for each row of z (CUDA tensor (R, 3N) of the engine's
    precision; positions already set).  Iterates until the relative change of
    every row's estimate is below `tol` or `max_iter`.  Returns (y, iterations)."""
    R, n3 = z.shape
    dtype = z.dtype
    znorm = torch.linalg.norm(z, dim=1, keepdim=True)
    safe = torch.where(znorm > 0, znorm, torch.ones_like(znorm))
    V = [z / safe]
    alphas, betas = [], []
    w = torch.empty_like(z)
    y_prev = None
    for j in range(max_iter):
        engine.apply(V[j], w)
        a = (V[j] * w).sum(dim=1)
        w = w - a[:, None] * V[j]
        if j > 0:
            w = w - betas[-1][:, None] * V[j - 1]
        if reorthogonalize:
            for Vk in V:
                w = w - (Vk * w).sum(dim=1, keepdim=True) * Vk
        alphas.append(a)
        b = torch.linalg.norm(w, dim=1)
        coeff = _sqrt_tridiag_e1(torch.stack(alphas, 1).double(),
                                 torch.stack(betas, 1).double() if betas else
                                 torch.zeros(R, 0, dtype=torch.float64, device=z.device))
        Vm = torch.stack(V, 1).double()  # (R, m, 3N)
        y = (znorm.double() * (Vm * coeff).sum(dim=1)).to(dtype)
        if y_prev is not None:
            rel = torch.linalg.norm(y - y_prev, dim=1) / torch.clamp(
                torch.linalg.norm(y, dim=1), min=1e-300)
            if bool((rel < tol).all()):
                return y, j + 1
        y_prev = y
        if bool((b <= 1e-12 * torch.clamp(znorm[:, 0], min=1e-300)).all()):
            return y, j + 1  # invariant subspace: exact
        betas.append(b)
        V.append(w / torch.where(b > 0, b, torch.ones_like(b))[:, None])
        w = torch.empty_like(z)
    return y_prev, max_iter


def brownian_displacements(engine, forces, dt: float, kT: float = 1.0,
                           mobility_scale: float = 1.0, generator=None, tol: float = 1e-4,
                           max_iter: int = 60):
    """Displacements dx = s M F dt + sqrt(2 kT dt s) M^{1/2} xi for R
    independent samples (rows of `forces`, CUDA (R, 3N)); s = mobility_scale
    converts the operator's units (mobility x 6 pi eta) to a mobility
    (s = 1 / (6 pi eta)).  Returns (dx, lanczos iterations)."""
    drift = torch.zeros_like(forces)
    engine.apply(forces, drift)
    xi = torch.randn(forces.shape, generator=generator, device=forces.device,
                     dtype=forces.dtype)
    noise, iters = sqrt_mobility_apply(engine, xi, tol=tol, max_iter=max_iter)
    return mobility_scale * dt * drift + (2.0 * kT * dt * mobility_scale) ** 0.5 * noise, iters
