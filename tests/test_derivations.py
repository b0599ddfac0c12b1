"""CPU checks of two derivations the CUDA kernels rely on (numpy FFT as the
reference; no GPU):

* the fused z-FFT kernel applies, on the kx = 0 and K/2 planes, the influence
  tensor averaged with its mirror, I_sym = (I(k) + I(-k)) / 2, instead of forming
  the Hermitian part of I(k) g afterwards; for the Hermitian spectrum g of real
  data both are equal under the reference's Nyquist convention (the index K/2
  maps to +pi K / L), and I_sym is I with the couplings between a Nyquist or zero
  axis and any other axis kept only where the kernel's sign rule says so;
* the one-pass 2D transforms split a real row into K/2 complex values, split the
  transform back into the half spectrum, pack the kx = 0 and K/2 columns into one
  complex column, and invert all of it.
"""
import numpy as np
import pytest


def _wav(i, K):
    # the reference's convention (old-version/spme.c:96-107): i <= K/2 -> +i
    return i if i <= K // 2 else i - K


@pytest.mark.parametrize("K", [8, 9, 10])
def test_mirror_averaged_influence_is_the_hermitian_part(K):
    rng = np.random.default_rng(K)
    g = np.fft.rfftn(rng.standard_normal((3, K, K, K)), axes=(1, 2, 3))  # [c][kz][ky][kx]
    Kh = K // 2 + 1
    kz = np.array([_wav(i, K) for i in range(K)], float)[:, None, None]
    ky = np.array([_wav(i, K) for i in range(K)], float)[None, :, None]
    kx = np.arange(Kh, dtype=float)[None, None, :]
    kzb, kyb, kxb = np.broadcast_arrays(kz, ky, kx)
    k2 = kxb ** 2 + kyb ** 2 + kzb ** 2
    k2[0, 0, 0] = 1.0
    m2 = np.exp(-0.1 * k2) + 0.3 * np.cos(k2)  # scalar factors depend on |k| only
    c = m2 / k2
    kv = [kxb, kyb, kzb]
    B = [[(m2 if i == j else 0.0) - c * kv[i] * kv[j] for j in range(3)] for i in range(3)]

    def apply(b):
        return np.stack([sum(b[i][j] * g[j] for j in range(3)) for i in range(3)])

    Ig = apply(B)
    # Hermitian part over (ky, kz) <-> (-ky, -kz) on the kx = 0 and (even K) K/2 planes
    planes = [0] + ([K // 2] if K % 2 == 0 else [])
    neg = (-np.arange(K)) % K
    H = Ig.copy()
    for p in planes:
        P = Ig[:, :, :, p]
        H[:, :, :, p] = 0.5 * (P + np.conj(P[:, neg][:, :, neg]))
    # the kernel's rule: s = +1 for a zero or Nyquist index, -1 otherwise (s_x = +1
    # on these planes); the ij coupling survives where s_i s_j = +1
    iy = np.arange(K)[None, :, None]
    iz = np.arange(K)[:, None, None]
    sy = (iy == 0) | ((K % 2 == 0) & (iy == K // 2))
    sz = (iz == 0) | ((K % 2 == 0) & (iz == K // 2))
    on = np.zeros(k2.shape, bool)
    for p in planes:
        on[:, :, p] = True
    keep = {(0, 1): sy, (0, 2): sz, (1, 2): sy == sz}
    Bs = [[B[i][j] for j in range(3)] for i in range(3)]
    for (i, j), kp in keep.items():
        drop = on & ~np.broadcast_to(kp, k2.shape)
        Bs[i][j] = Bs[j][i] = np.where(drop, 0.0, B[i][j])
    assert np.abs(apply(Bs) - H).max() <= 1e-12 * np.abs(H).max()


def _w(e, n):
    return np.exp(-2j * np.pi * e / n)


@pytest.mark.parametrize("K", [128, 160, 256])
def test_one_pass_2d_decomposition(K):
    rng = np.random.default_rng(K)
    M, NC = K // 2, K // 4
    x = rng.standard_normal((K, K))  # [y][x]
    # forward: rows as M complex values, M-point transform, split
    Z = np.fft.fft(x[:, 0::2] + 1j * x[:, 1::2], axis=1)
    cols = [np.zeros((K, NC), complex), np.zeros((K, NC), complex)]  # the two CTAs' columns
    for j in range(M // 2):
        if j == 0:
            z0, zh = Z[:, 0], Z[:, M // 2]
            cols[0][:, 0] = (z0.real + z0.imag) + 1j * (z0.real - z0.imag)  # X[0] + i X[M]
            cols[1][:, 0] = np.conj(zh)  # X[M/2]
        else:
            zk, zm = Z[:, j], np.conj(Z[:, M - j])
            e = 0.5 * (zk + zm)
            t = _w(j, K) * (-0.5j) * (zk - zm)
            cols[0][:, j] = e + t  # X[j]
            cols[1][:, M // 2 - j] = np.conj(e - t)  # X[M - j]
    F = [np.fft.fft(cc, axis=0) for cc in cols]
    half = np.zeros((K, M + 1), complex)
    C0 = F[0][:, 0]
    C0m = np.conj(C0[(-np.arange(K)) % K])
    half[:, 0], half[:, M] = 0.5 * (C0 + C0m), (C0 - C0m) / 2j
    half[:, 1:M // 2] = F[0][:, 1:]
    half[:, M // 2:M] = F[1]
    ref = np.fft.rfft2(x)
    assert np.abs(half - ref).max() <= 1e-10 * np.abs(ref).max()
    # inverse: packed column, K-point inverse, rows back, packing, M-point inverse
    colsi = [np.zeros((K, NC), complex), np.zeros((K, NC), complex)]
    colsi[0][:, 0] = ref[:, 0] + 1j * ref[:, M]
    colsi[0][:, 1:] = ref[:, 1:M // 2]
    colsi[1][:, :] = ref[:, M // 2:M]
    T = [np.fft.ifft(cc, axis=0) * K for cc in colsi]
    X = np.zeros((K, M + 1), complex)
    X[:, 0], X[:, M] = T[0][:, 0].real, T[0][:, 0].imag
    X[:, 1:M // 2], X[:, M // 2:M] = T[0][:, 1:], T[1]
    out = np.zeros((K, K))
    for y in range(K):
        Zp = np.zeros(M, complex)
        for j in range(M // 2):
            if j == 0:
                x0, xm = X[y, 0].real, X[y, M].real
                Zp[0] = (x0 + xm) + 1j * (x0 - xm)
                Zp[M // 2] = 2 * np.conj(X[y, M // 2])
            else:
                xk, xm = X[y, j], np.conj(X[y, M - j])
                iu = 1j * (xk - xm) * np.conj(_w(j, K))
                Zp[j], Zp[M - j] = (xk + xm) + iu, np.conj((xk + xm) - iu)
        z = np.fft.ifft(Zp) * M
        out[y, 0::2], out[y, 1::2] = z.real, z.imag
    assert np.abs(out - x * K * K).max() <= 1e-9 * K * K
