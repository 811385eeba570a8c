"""Algebra the device kernels rely on, restated in FP64 NumPy on the host and checked against the oracle.

1. The one-sweep Lanczos recurrence of the FP32 GPU path.

The device path (``gato_gb300/csrc/lanczos.cu``: ``k_fz_sweep``, ``k_fz_form``, ``k_fz_post2``)
applies the operator to the three-term vector w^_(j-1) *before* its Gram-Schmidt correction and
recovers F v_j from the Lanczos relation F V = V T~, so each step reads the basis once:

* sweep j:  v_j = (w^ - V c) / beta,  u_j = F v_j = (z - V g - g_j v_j) / beta,  z = F w^,
            a_k = <v_k, u_j>,  d_k = <v_k, v_j>  (k <= j);
* form:     alpha_j = a_j - beta_(j-1) d_(j-1),
            c_k = a_k - beta_(j-1) <v_k, v_(j-1)> - alpha_j d_k  (the coefficients of w^_j),
            w^_j = u_j - beta_(j-1) v_(j-1) - alpha_j v_j;
* post:     beta_j^2 = |w^_j|^2 - |c|^2  (Pythagoras),
            g_i = sum_k T~_ik c_k  with  T~ = tridiag(beta, alpha, beta) + the earlier correction rows.

In exact arithmetic this is the reference's Lanczos with full modified Gram-Schmidt
reorthogonalisation (``solvers/lanczos.py:110-206``). The tests run both in FP64 on a small
oscillator and hold the tridiagonal coefficients and eigenvalues to rounding-level agreement, so
the algebra of the GPU recurrence is checked apart from its FP32 arithmetic.

2. The spectral (Parseval) form of the FP64 energy pass, against the oracle's Hockney solve.
"""
import math

import numpy as np
import pytest

from oracle import gato_np as o


def one_sweep_lanczos(H, psi0, m):
    grid = H.grid
    dV = grid.h ** 3

    def ip(a, b):
        return dV * float(np.dot(a, b))

    def F(x):
        return H.apply(x.reshape(grid.shape)).ravel()

    n = psi0.size
    V = np.zeros((m, n))
    v0 = psi0.ravel() / math.sqrt(ip(psi0.ravel(), psi0.ravel()))
    wh, z = v0.copy(), F(v0)              # step 0 takes v_0 itself: beta = 1, c = g = 0
    c, g, beta_in = np.zeros(0), np.zeros(1), 1.0
    alphas, betas = np.zeros(m), np.zeros(m)
    Cm = np.zeros((m, m))
    dprev = np.zeros(m)
    for j in range(m):
        bi = 1.0 / beta_in if beta_in > 0 else 0.0
        vj = (wh - V[:j].T @ c) * bi
        uj = (z - V[:j].T @ g[:j] - g[j] * vj) * bi
        V[j] = vj
        a = np.array([ip(V[k], uj) for k in range(j + 1)])
        d = np.array([ip(V[k], vj) for k in range(j + 1)])
        beta_p = betas[j - 1] if j > 0 else 0.0
        alpha = a[j] - beta_p * (d[j - 1] if j > 0 else 0.0)
        alphas[j] = alpha
        for k in range(j + 1):
            bk = 0.0 if j == 0 else (dprev[k] if k < j else d[j - 1])
            Cm[j, k] = a[k] - beta_p * bk - alpha * d[k]
        dprev[: j + 1] = d
        wh = uj - beta_p * (V[j - 1] if j > 0 else vj) - alpha * vj
        c = Cm[j, : j + 1].copy()
        b2 = ip(wh, wh) - float(c @ c)
        beta_in = math.sqrt(b2) if b2 > 0 else 0.0
        betas[j] = beta_in
        g = np.zeros(j + 2)
        for i in range(j + 2):
            gi = 0.0
            if i + 1 <= j:
                gi += c[i + 1] * betas[i]
            if i <= j:
                gi += c[i] * alphas[i]
            if i >= 1:
                gi += c[i - 1] * betas[i - 1]
            for k in range(i, j + 1):
                gi += c[k] * Cm[k, i]
            g[i] = gi
        if j + 1 < m:
            z = F(wh)
    return alphas, betas, V


def _tridiag_eigs(alphas, betas):
    m = len(alphas)
    T = np.diag(alphas) + np.diag(betas[: m - 1], 1) + np.diag(betas[: m - 1], -1)
    return np.linalg.eigvalsh(T)


@pytest.fixture(scope="module")
def oscillator():
    g = o.Grid3D(14, 12.0)
    X, Y, Z = np.meshgrid(*(3 * [-g.L / 2 + (np.arange(g.N) + 0.5) * g.h]), indexing="ij")
    V = 0.5 * (X * X + 1.3 * Y * Y + 1.7 * Z * Z)    # anisotropic: no degenerate levels
    H = o.Hamiltonian(g, V, order=4)
    psi0 = np.random.default_rng(5).uniform(0.0, 1.0, g.shape)
    return H, psi0


def test_one_sweep_recurrence_matches_mgs_lanczos(oscillator):
    H, psi0 = oscillator
    m = 60
    ref = o.lanczos(H, psi0, n_iters=m, n_eigenstates=4)
    alphas, betas, V = one_sweep_lanczos(H, psi0, m)
    # the leading coefficients agree to rounding; late ones are forward-unstable after Ritz convergence
    assert np.max(np.abs(alphas[:8] - ref.alphas[:8])) < 1e-11 * np.max(np.abs(ref.alphas[:8]))
    assert np.max(np.abs(betas[:8] - ref.betas[:8])) < 1e-11 * np.max(np.abs(ref.betas[:8]))
    e_one = _tridiag_eigs(alphas, betas)[:4]
    e_ref = np.asarray(ref.eigenvalues)[:4]
    assert np.max(np.abs(e_one - e_ref)) < 1e-10
    # the basis stays orthonormal to rounding (the relation replaces a second reorthogonalisation pass)
    G = (H.grid.h ** 3) * (V @ V.T)
    assert np.max(np.abs(G - np.eye(m))) < 1e-10


def test_one_sweep_ground_state_energy_is_an_upper_bound_that_converges(oscillator):
    H, psi0 = oscillator
    e_short = _tridiag_eigs(*one_sweep_lanczos(H, psi0, 20)[:2])[0]
    e_long = _tridiag_eigs(*one_sweep_lanczos(H, psi0, 60)[:2])[0]
    # Rayleigh-Ritz: more Krylov vectors never raise the lowest Ritz value
    assert e_long <= e_short + 1e-12


def test_spectral_energy_identity_of_the_fp64_energy_pass():
    """The FP64 energy pass (``k_cols_fe``) forms a Hartree-type energy from the x-forward spectrum
    alone: for two real densities a, b packed as F = a + i b on the doubled grid, with the kernel
    spectrum G^ real and even, sum_k G^_k |F^_k|^2 / M^3 * dV^2 = <a, J[a]> + <b, J[b]> (Parseval for
    the circular convolution; the a-b cross terms cancel between k and -k). Checked on the host against
    the oracle's Hockney solve (``poisson.py:47-79``)."""
    N, h = 12, 0.4
    g = o.Grid3D(N, N * h)
    rng = np.random.default_rng(17)
    a, b = rng.standard_normal(g.shape), rng.standard_normal(g.shape)
    eps = h / 2
    dV = g.h ** 3
    direct = dV * float(np.sum(a * o.hartree_potential(a, g, eps))) + dV * float(np.sum(b * o.hartree_potential(b, g, eps)))
    M = 2 * N
    F = np.zeros((M, M, M), dtype=complex)
    F[:N, :N, :N] = a + 1j * b
    Gh = np.fft.fftn(o._coulomb_kernel(N, h, eps))
    assert np.max(np.abs(Gh.imag)) < 1e-9 * np.max(np.abs(Gh.real))   # real and even
    spectral = float(np.sum(Gh.real * np.abs(np.fft.fftn(F)) ** 2)) / M ** 3 * dV * dV
    assert abs(spectral - direct) < 1e-12 * abs(direct)
