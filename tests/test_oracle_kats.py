"""Pin the CPU oracle to the reference's own known-answer tests.

The reference (ezequielgarcia/gato) ships no golden arrays; its tests assert
analytic invariants. Each test here restates one of those invariants against
``oracle.gato_np`` with the reference's grid sizes and tolerances, citing the
reference test it follows (paths relative to the reference's ``tests/``).
"""
import math

import numpy as np
import pytest
import scipy.fft
import scipy.special

from oracle import gato_np as o


def _periodic_coords(N, L):
    h = L / N
    a = np.arange(N) * h
    X, Y, Z = np.meshgrid(a, a, a, indexing="ij")
    return X, Y, Z, h


# ---- operators (test_laplacian.py, test_laplacian_order4.py) --------------

def test_order2_plane_wave_eigenvector():            # test_laplacian.py:24-38
    X, Y, Z, h = _periodic_coords(32, 4.0)
    kx, ky, kz = 2 * np.pi / 4.0 * np.array([1.0, 2.0, -1.0])
    psi = np.exp(1j * (kx * X + ky * Y + kz * Z))
    lap = o.laplacian(psi, h, "periodic")
    eig = -2.0 * ((1 - np.cos(kx * h)) + (1 - np.cos(ky * h)) + (1 - np.cos(kz * h))) / h ** 2
    assert np.max(np.abs(lap - eig * psi)) < 1e-10


def test_order4_plane_wave_eigenvalue():             # test_laplacian_order4.py:46-57
    X, Y, Z, h = _periodic_coords(32, 4.0)
    ks = 2 * np.pi / 4.0 * np.array([1.0, 2.0, -1.0])
    psi = np.exp(1j * (ks[0] * X + ks[1] * Y + ks[2] * Z))
    lam = sum(30 / 12 - 32 / 12 * np.cos(k * h) + 2 / 12 * np.cos(2 * k * h) for k in ks) / h ** 2
    assert np.max(np.abs(o.laplacian(psi, h, "periodic", 4) + lam * psi)) < 1e-10


def test_convergence_rates():                        # test_laplacian.py:41-58, order4:60-84
    L = 10.0
    k = 2 * np.pi / L
    errs = {2: [], 4: []}
    for N in (16, 32, 64):
        X, Y, Z, h = _periodic_coords(N, L)
        psi = np.exp(1j * k * (X + Y + Z))
        for order in (2, 4):
            lap = o.laplacian(psi, h, "periodic", order)
            errs[order].append(abs(float((-lap[0, 0, 0] / psi[0, 0, 0]).real) - 3 * k * k))
    assert errs[2][1] < errs[2][0] / 3.5 and errs[2][2] < errs[2][1] / 3.5
    assert errs[4][1] < errs[4][0] / 12 and errs[4][2] < errs[4][1] / 12
    assert errs[4][-1] < errs[2][-1] * 1e-2


@pytest.mark.parametrize("order", [2, 4])
def test_dirichlet_hermitian(order):                 # test_laplacian.py:61-72, order4:87-98
    g = o.Grid3D(16, 5.0)
    rng = np.random.default_rng(order)
    phi, psi = rng.standard_normal(g.shape), rng.standard_normal(g.shape)
    lhs = np.sum(phi * o.laplacian(psi, g.h, "dirichlet", order))
    rhs = np.sum(o.laplacian(phi, g.h, "dirichlet", order) * psi)
    assert abs(lhs - rhs) < 1e-8


def test_particle_in_box_converges():                # test_laplacian.py:75-106
    L = 6.0
    E_exact = 3 * (np.pi / L) ** 2 / 2
    errs = []
    for N in (32, 64, 128):
        g = o.Grid3D(N, L)
        X, Y, Z = g.coords()
        psi = np.cos(np.pi * X / L) * np.cos(np.pi * Y / L) * np.cos(np.pi * Z / L)
        E = np.sum(psi * o.kinetic(psi, g.h, "dirichlet")) / np.sum(psi * psi)
        errs.append(abs(E - E_exact))
    assert errs[1] < errs[0] and errs[2] < errs[1] and errs[2] / E_exact < 1e-2


def test_order4_gaussian_kinetic():                  # test_laplacian_order4.py:101-109
    g = o.Grid3D(48, 10.0)
    X, Y, Z = g.coords()
    psi = o.normalize(np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / 2), g)
    T = o.inner_product(psi, o.kinetic(psi, g.h, "dirichlet", 4), g).real
    assert abs(T - 0.75) < 5e-3


def test_bad_order_and_boundary_raise():             # test_laplacian.py:121-127, order4:112-119
    psi = np.ones((8, 8, 8))
    with pytest.raises(ValueError):
        o.laplacian(psi, 0.25, boundary="mystery")
    for bad in (3, 6):
        with pytest.raises(ValueError):
            o.laplacian(psi, 0.25, order=bad)


# ---- hamiltonian (test_hamiltonian.py) -------------------------------------

def test_hamiltonian_invariants():                   # test_hamiltonian.py:10-44
    g = o.Grid3D(16, 5.0)
    psi = np.random.default_rng(0).standard_normal(g.shape)
    H0 = o.Hamiltonian(g, o.constant(g, 0.0))
    assert np.max(np.abs(H0.apply(psi) - o.kinetic(psi, g.h))) < 1e-12
    g = o.Grid3D(16, 6.0)
    X, Y, Z = g.coords()
    H = o.Hamiltonian(g, o.harmonic_oscillator(g, 1.0))
    gau = np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / 2)
    assert abs(H.rayleigh(gau) - H.rayleigh(7.3 * gau)) < 1e-10
    g = o.Grid3D(48, 10.0)
    X, Y, Z = g.coords()
    H = o.Hamiltonian(g, o.harmonic_oscillator(g, 1.0))
    E = H.rayleigh(o.normalize(np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / 2), g))
    assert abs(E - 1.5) / 1.5 < 0.01


# ---- poisson (test_poisson.py) ---------------------------------------------

def _gaussian(g, alpha, center=(0.0, 0.0, 0.0)):
    X, Y, Z = g.coords()
    r2 = (X - center[0]) ** 2 + (Y - center[1]) ** 2 + (Z - center[2]) ** 2
    return (alpha / np.pi) ** 1.5 * np.exp(-alpha * r2)


def test_gaussian_hartree_energy():                  # test_poisson.py:27-38
    g = o.Grid3D(48, 10.0)
    rho = _gaussian(g, 0.5)
    assert abs(o.integrate(rho, g) - 1.0) < 1e-4
    E_exact = 0.5 * math.sqrt(2 * 0.5 / math.pi)
    assert abs(o.hartree_energy(rho, g) - E_exact) / E_exact < 1e-2


def test_hartree_far_field():                        # test_poisson.py:41-57
    g = o.Grid3D(80, 10.0)
    J = o.hartree_potential(_gaussian(g, 0.5), g)
    r = g.radial()
    mask = (r > 2.5) & (r < 3.5)
    exact = scipy.special.erf(math.sqrt(0.5) * r) / np.where(r > 0, r, 1.0)
    assert np.max(np.abs(J[mask] - exact[mask])) < 5e-4


def test_hartree_linear_positive_and_scaling():      # test_poisson.py:60-90
    g = o.Grid3D(32, 8.0)
    r1, r2 = _gaussian(g, 0.8, (0.5, 0, 0)), _gaussian(g, 1.2, (-0.7, 0.3, 0))
    J1, J2 = o.hartree_potential(r1, g), o.hartree_potential(r2, g)
    assert np.max(np.abs(o.hartree_potential(1.3 * r1 - 0.4 * r2, g) - (1.3 * J1 - 0.4 * J2))) < 1e-10
    assert np.min(o.hartree_potential(_gaussian(g, 1.0), g)) > 0
    g = o.Grid3D(48, 10.0)
    ratio = o.hartree_energy(_gaussian(g, 2.0), g) / o.hartree_energy(_gaussian(g, 0.5), g)
    assert abs(ratio - 2.0) / 2.0 < 2e-2


def test_spectral_energy_identity():
    """The identity the FP64 energy pass rests on: the kernel spectrum is real and even, so for two
    real densities packed as F = a + i b the kernel-weighted power of F's spectrum on the doubled
    grid equals the sum of both Hartree-type energies (the cross terms cancel between k and -k)."""
    g = o.Grid3D(12, 5.0)
    N, M = g.N, 2 * g.N
    rng = np.random.default_rng(3)
    a, b = rng.standard_normal(g.shape), rng.standard_normal(g.shape)
    Gh = scipy.fft.fftn(o._coulomb_kernel(N, g.h, g.h / 2))
    assert np.max(np.abs(Gh.imag)) < 1e-9 * np.max(np.abs(Gh.real))
    ghat = Gh.real * g.dV / M ** 3
    F = np.zeros((M, M, M), complex)
    F[:N, :N, :N] = a + 1j * b
    spectral = g.dV * np.sum(ghat * np.abs(scipy.fft.fftn(F)) ** 2)
    direct = o.integrate(a * o.hartree_potential(a, g), g) + o.integrate(b * o.hartree_potential(b, g), g)
    assert abs(spectral - direct) < 1e-11 * abs(direct)


# ---- lanczos (test_lanczos.py) ----------------------------------------------

def test_lanczos_ho_ground_state():                  # test_lanczos.py:22-36
    g = o.Grid3D(32, 10.0)
    H = o.Hamiltonian(g, o.harmonic_oscillator(g), order=4)
    X, Y, Z = g.coords()
    res = o.lanczos(H, np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / 2), n_iters=60, n_eigenstates=4)
    assert abs(res.eigenvalues[0] - 1.5) < 1e-2


def test_lanczos_ho_ladder_and_orthonormality():     # test_lanczos.py:39-92
    g = o.Grid3D(40, 10.0)
    H = o.Hamiltonian(g, o.harmonic_oscillator(g), order=4)
    res = o.lanczos(H, np.random.default_rng(1).standard_normal(g.shape), n_iters=120, n_eigenstates=12)
    rungs = []
    for e in sorted(res.eigenvalues):
        if not rungs or abs(e - rungs[-1]) > 1e-2:
            rungs.append(e)
    assert len(rungs) >= 4
    for got, want in zip(rungs, [1.5, 2.5, 3.5, 4.5]):
        assert abs(got - want) < 5e-3
    g = o.Grid3D(24, 10.0)
    X, Y, Z = g.coords()
    H = o.Hamiltonian(g, o.harmonic_oscillator(g), order=4)
    res = o.lanczos(H, np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / 2) * (1 + 0.1 * (X + Y + Z)), 40, 3)
    S = np.einsum("xyzi,xyzj->ij", res.eigenstates, res.eigenstates) * g.dV
    assert np.max(np.abs(S - np.eye(3))) < 1e-6


def test_default_krylov_dim():                       # test_lanczos.py:115-151
    dims = [o.default_krylov_dim(N, 4) for N in (32, 48, 64, 96, 128)]
    assert dims == sorted(dims) and dims[-1] > dims[0]
    assert o.default_krylov_dim(64, 4) >= 80 and o.default_krylov_dim(96, 4) >= 120
    assert o.default_krylov_dim(128, 4) >= 160
    assert o.default_krylov_dim(40, 4) >= 120 and o.default_krylov_dim(8, 12) > 12
    assert o.default_krylov_dim(64, 1) == 80 and o.default_krylov_dim(96, 1) == 120


# ---- scf (test_scf.py) ------------------------------------------------------

def _ngauss(g, alpha):
    X, Y, Z = g.coords()
    return o.normalize((2 * alpha / np.pi) ** 0.75 * np.exp(-alpha * (X * X + Y * Y + Z * Z)), g)


def test_exchange_self_reduction():                  # test_scf.py:44-53
    g = o.Grid3D(32, 8.0)
    phi = _ngauss(g, 1.0)
    K = o.exchange_apply(phi, phi[..., None], g)
    assert np.max(np.abs(K - phi * o.hartree_potential(phi ** 2, g))) < 1e-12


def test_fock_zero_orbitals_is_core():               # test_scf.py:56-69
    g = o.Grid3D(24, 6.0)
    V = o.softened_coulomb(g, Z=2.0)
    F = o.RHFFock(g, V, np.zeros(g.shape + (1,)), np.zeros(g.shape), order=4)
    psi = _ngauss(g, 1.5)
    assert np.max(np.abs(F.apply(psi) - o.Hamiltonian(g, V, order=4).apply(psi))) < 1e-12


def test_single_orbital_energy_identity():           # test_scf.py:72-94
    g = o.Grid3D(32, 8.0)
    phi = _ngauss(g, 1.0)
    E = o.rhf_energy(phi[..., None], np.zeros(g.shape), g)
    rho1 = phi ** 2
    expected = (np.sum(rho1 * o.hartree_potential(rho1, g)) * g.dV
                + 2 * o.inner_product(phi, o.kinetic(phi, g.h, "dirichlet", 4), g))
    assert abs(E - expected) < 1e-10


@pytest.mark.slow
def test_helium_scf():                               # test_scf.py:97-126
    g = o.Grid3D(64, 10.0)
    res = o.scf_rhf(o.softened_coulomb(g, Z=2.0), g, 1, max_iters=25, tol=1e-6, mixing=0.7,
                    order=4, lanczos_iters=40)
    assert res.converged and res.energy > -3.0 and abs(res.energy + 2.599) < 0.010


def test_block_fock_matches_matvec():
    """The pair-symmetric block Fock apply equals scf.py:88-111 per orbital."""
    g = o.Grid3D(16, 8.0)
    rng = np.random.default_rng(3)
    orbs = rng.standard_normal((3,) + g.shape)
    V = rng.standard_normal(g.shape)
    F = o.RHFFock(g, np.zeros(g.shape), np.moveaxis(orbs, 0, -1), V, order=4)
    blk = o.fock_apply_block(orbs, V, g)
    for i in range(3):
        assert np.max(np.abs(blk[i] - F.apply(orbs[i]))) < 1e-10 * np.max(np.abs(blk[i]))


# ---- pseudopotentials (test_pseudopotentials.py) ---------------------------

ALL = [o.HYDROGEN_HGH, o.LITHIUM_HGH, o.OXYGEN_HGH, o.CHLORINE_HGH]


@pytest.mark.parametrize("params", ALL, ids=lambda p: p.symbol)
def test_hgh_local_tail_and_origin(params):          # test_pseudopotentials.py:39-113
    g = o.Grid3D(64, 20.0)
    nuc = o.Nuclei(np.zeros((1, 3)), np.array([params.Z_ion]))
    V = o.hgh_local_potential(nuc, (params,), g).ravel()
    r = g.radial().ravel()
    i = int(np.argmin(np.abs(r - 5.0)))
    assert abs(V[i] + params.Z_ion / r[i]) < 1e-6
    g = o.Grid3D(32, 3.0)
    V = o.hgh_local_potential(nuc, (params,), g).ravel()
    r = g.radial().ravel()
    i = int(np.argmin(r))
    rm = r[i]
    rho2 = (rm / params.r_loc) ** 2
    c1, c2, c3, c4 = params.c
    exp = (-params.Z_ion * math.erf(rm / (math.sqrt(2) * params.r_loc)) / rm
           + math.exp(-0.5 * rho2) * (c1 + c2 * rho2 + c3 * rho2 ** 2 + c4 * rho2 ** 3))
    assert abs(V[i] - exp) < 1e-9


@pytest.mark.parametrize("ell,i_idx,r_ell", [(0, 1, 0.22178614), (0, 1, 0.5), (1, 1, 0.4), (0, 2, 0.3)])
def test_projector_normalisation(ell, i_idx, r_ell):   # test_pseudopotentials.py:120-138
    r = np.linspace(1e-6, 8.0 * r_ell, 20000)
    p = o._projector_radial(r, ell, i_idx, r_ell)
    assert abs(np.trapezoid(p * p * r * r, r) - 1.0) < 1e-4


@pytest.mark.parametrize("params", [o.OXYGEN_HGH, o.CHLORINE_HGH, o.LITHIUM_HGH], ids=lambda p: p.symbol)
def test_nonlocal_hermitian(params):                 # test_pseudopotentials.py:145-224
    g = o.Grid3D(40, 10.0)
    nuc = o.Nuclei(np.zeros((1, 3)), np.array([params.Z_ion]))
    rng = np.random.default_rng(0)
    phi, psi = rng.standard_normal(g.shape), rng.standard_normal(g.shape)
    a = o.inner_product(phi, o.hgh_nonlocal_apply(psi, nuc, (params,), g), g)
    b = o.inner_product(o.hgh_nonlocal_apply(phi, nuc, (params,), g), psi, g)
    assert abs(a - b) < 1e-9 * (abs(a) + abs(b) + 1.0)


def test_lookup():                                   # test_pseudopotentials.py:227-233
    assert o.lookup("O") is o.OXYGEN_HGH and o.lookup("Cl") is o.CHLORINE_HGH
    with pytest.raises(KeyError):
        o.lookup("Xx")


# ---- geometry (test_geometry.py, test_multicenter_potential.py) -------------

def test_nuclear_repulsion_and_forces():             # test_geometry.py:46-80
    for R in (1.0, 2.0, 3.5):
        assert o.nuclear_repulsion(o.diatomic_along_z(R, 1.0)) == pytest.approx(1 / R, rel=1e-10)
    assert o.nuclear_repulsion(o.Nuclei(np.zeros((1, 3)), np.array([1.0]))) == 0.0
    F = -o.nuclear_repulsion_grad(o.diatomic_along_z(2.0, 1.0))
    assert F[0, 2] == pytest.approx(-0.25, rel=1e-12) and F[1, 2] == pytest.approx(0.25, rel=1e-12)
    assert np.allclose(F[:, :2], 0.0, atol=1e-14)


def test_multicenter_superposition():               # test_multicenter_potential.py:11-44
    g = o.Grid3D(24, 8.0)
    one = o.Nuclei(np.zeros((1, 3)), np.array([1.0]))
    assert np.allclose(o.multi_center_softened_coulomb(one, g, 0.3), o.softened_coulomb(g, 1.0, 0.3), atol=1e-14)
    both = o.Nuclei(np.array([[0, 0, -1.0], [0, 0, 1.0]]), np.array([1.0, 1.0]))
    Va = o.softened_coulomb(g, 1.0, 0.3, (0, 0, -1.0))
    Vb = o.softened_coulomb(g, 1.0, 0.3, (0, 0, 1.0))
    assert np.allclose(o.multi_center_softened_coulomb(both, g, 0.3), Va + Vb, atol=1e-12)


# ---- forces: the analytic restatement of jax.grad vs central differences ----

def test_bo_gradient_matches_finite_difference():    # test_water.py:52-80 (rel 1e-3 / abs 1e-4)
    g = o.Grid3D(24, 12.0)
    nuc = o.water_initial_geometry(1.85, 104.0)
    elements = o.water_hgh_elements()
    rng = np.random.default_rng(5)
    X, Y, Z = g.coords()
    # fixed smooth orbitals stand in for converged ones: the identity tested
    # is d/dR of the R-dependent energy at fixed orbitals.
    orbs = np.stack([np.exp(-0.6 * ((X - a) ** 2 + (Y - b) ** 2 + (Z - c) ** 2))
                     for a, b, c in rng.uniform(-0.8, 0.8, (4, 3))], axis=-1)
    grad = o.bo_grad_positions(nuc.positions, nuc.charges, orbs, elements, g)
    d = 1e-3
    for atom, ax in [(1, 2), (0, 0), (2, 1), (0, 2)]:
        p, m = nuc.positions.copy(), nuc.positions.copy()
        p[atom, ax] += d
        m[atom, ax] -= d
        fd = (o.bo_energy_position_part(p, nuc.charges, orbs, elements, g)
              - o.bo_energy_position_part(m, nuc.charges, orbs, elements, g)) / (2 * d)
        assert grad[atom, ax] == pytest.approx(fd, rel=1e-3, abs=1e-4)
    # bo_energy's R-independent terms cancel in a difference: check one pair
    p, m = nuc.positions.copy(), nuc.positions.copy()
    p[1, 2] += d
    m[1, 2] -= d
    full = (o.bo_energy(p, nuc.charges, orbs, elements, g) - o.bo_energy(m, nuc.charges, orbs, elements, g)) / (2 * d)
    assert grad[1, 2] == pytest.approx(full, rel=1e-3, abs=1e-4)


def test_adam_matches_published_update():
    """Adam (Kingma & Ba, optax defaults): the first step is -lr * sign(g)."""
    opt = o.Adam(0.02)
    g = np.array([[0.3, -2.0, 1e-3]])
    u = opt.update(g)
    assert np.allclose(u, -0.02 * g / (np.abs(g) + 1e-8), rtol=1e-12)


def test_softened_coulomb_grad_matches_finite_difference():
    """The analytic d/dR int rho V_ext of the H2 force path against a central difference."""
    g = o.Grid3D(24, 8.0)
    X, Y, Z = g.coords()
    rho = np.exp(-0.6 * (X * X + Y * Y + (Z - 0.2) ** 2))
    pos = np.array([[0.0, 0.1, -0.7], [0.05, 0.0, 0.7]])
    nuc = o.Nuclei(pos, np.array([1.0, 1.0]))
    ga = o.multi_center_softened_coulomb_grad(nuc, g, rho, 0.3)
    d = 1e-4
    for k in range(2):
        for c in range(3):
            pp, pm = pos.copy(), pos.copy()
            pp[k, c] += d
            pm[k, c] -= d
            ep = np.sum(rho * o.multi_center_softened_coulomb(o.Nuclei(pp, nuc.charges), g, 0.3)) * g.dV
            em = np.sum(rho * o.multi_center_softened_coulomb(o.Nuclei(pm, nuc.charges), g, 0.3)) * g.dV
            assert abs(ga[k, c] - (ep - em) / (2 * d)) < 1e-7
