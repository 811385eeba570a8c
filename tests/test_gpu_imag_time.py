"""Imaginary-time propagation, the hydrogen driver and the observables (reference:
solvers/imag_time.py, physics/hydrogen.py, observables.py; tests/test_hydrogen.py,
tests/test_lanczos.py:95-113 and tests/test_observables.py)."""
import numpy as np
import pytest
import torch

from oracle import gato_np as o

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")


@pytest.mark.parametrize("order", [2, 4])
def test_imag_time_matches_oracle(order):
    from gato_gb300.grid import Grid3D
    from gato_gb300.hamiltonian import Hamiltonian
    from gato_gb300.potentials import harmonic_oscillator
    from gato_gb300.solvers.imag_time import imaginary_time
    og, g = o.Grid3D(32, 10.0), Grid3D(32, 10.0)
    X, Y, Z = og.coords()
    psi0 = np.exp(-0.3 * ((X - 0.4) ** 2 + Y ** 2 + (Z + 0.2) ** 2)) * (1 + 0.2 * X)
    Vh = 0.5 * (X * X + Y * Y + Z * Z)
    ref_psi, ref_steps, ref_E = o.imaginary_time_logged(o.Hamiltonian(og, Vh, order=order), psi0, n_steps=301,
                                                        log_every=50)
    psi, hist = imaginary_time(Hamiltonian(g, harmonic_oscillator(g), order=order),
                               torch.tensor(psi0, device="cuda"), n_steps=301, log_every=50)
    assert hist.steps == ref_steps == [0, 50, 100, 150, 200, 250, 300]
    assert np.max(np.abs(np.array(hist.energies) - np.array(ref_E))) < 1e-12
    assert np.max(np.abs(psi.cpu().numpy() - ref_psi)) < 1e-11 * np.max(np.abs(ref_psi))


def test_imag_time_fp32_and_edge_cases():
    from gato_gb300.grid import Grid3D
    from gato_gb300.hamiltonian import Hamiltonian
    from gato_gb300.potentials import harmonic_oscillator
    from gato_gb300.solvers.imag_time import imaginary_time
    g = Grid3D(32, 10.0)
    V = harmonic_oscillator(g)
    X, Y, Z = g.coords()
    psi0 = torch.exp(-0.3 * (X * X + Y * Y + Z * Z)).contiguous()
    p64, h64 = imaginary_time(Hamiltonian(g, V, order=2), psi0, n_steps=400, log_every=100)
    p32, h32 = imaginary_time(Hamiltonian(g, V.float(), order=2), psi0.float(), n_steps=400, log_every=100)
    assert abs(h32.energies[-1] - h64.energies[-1]) < 1e-5
    assert all(a >= b - 1e-12 for a, b in zip(h64.energies, h64.energies[1:]))   # monotone decrease
    p0, h0 = imaginary_time(Hamiltonian(g, V, order=2), psi0, n_steps=0)
    assert h0.steps == [] and h0.energies == []
    assert abs(float((p0 * p0).sum()) * g.dV - 1.0) < 1e-12   # normalised, not stepped
    with pytest.raises(ValueError):
        imaginary_time(Hamiltonian(g, V, order=3), psi0, n_steps=5)
    # the step is a replayed CUDA graph: one counted launch per replay instead of four kernels
    from gato_gb300 import _lib
    n0 = _lib.launch_count()
    imaginary_time(Hamiltonian(g, V, order=2), psi0, n_steps=200, log_every=1000)
    assert _lib.launch_count() - n0 < 2 * 200


def test_hydrogen_imag_time_converges():
    """tests/test_hydrogen.py:11-21."""
    from gato_gb300.physics.hydrogen import solve_hydrogen
    res = solve_hydrogen(N=40, L=10.0, n_steps=1500, verbose=False)
    assert -0.55 < res.energy < -0.44, res.energy
    assert abs(res.virial_ratio - 1.0) < 0.08


def test_hydrogenic_ions_scale_as_minus_z_squared_over_two():
    """tests/test_hydrogen.py:24-49."""
    from gato_gb300.physics.hydrogen import solve_hydrogen
    for Z, L in ((1.0, 10.0), (2.0, 6.0), (3.0, 4.0)):
        res = solve_hydrogen(N=48, L=L, Z=Z, n_steps=1500, order=4, verbose=False)
        assert abs((res.energy + 0.5 * Z * Z) / (0.5 * Z * Z)) < 0.08, (Z, res.energy)
        assert abs(res.virial_ratio - 1.0) < 0.08


def test_lanczos_vs_imag_time_hydrogen_ground_state():
    """tests/test_lanczos.py:95-113 (the hydrogenic start replaces the JAX-keyed one)."""
    from gato_gb300.ansatz import init_grid_ansatz
    from gato_gb300.grid import Grid3D
    from gato_gb300.hamiltonian import Hamiltonian
    from gato_gb300.potentials import softened_coulomb
    from gato_gb300.solvers.imag_time import imaginary_time
    from gato_gb300.solvers.lanczos import lanczos
    g = Grid3D(40, 10.0)
    H = Hamiltonian(g, softened_coulomb(g, Z=1.0), order=4)
    psi0 = init_grid_ansatz(g, 2, init="hydrogenic", Z=1.0)
    E_lz = float(lanczos(H, psi0, n_iters=60, n_eigenstates=1).eigenvalues[0])
    _, hist = imaginary_time(H, psi0, n_steps=1500, log_every=500)
    assert abs(E_lz - hist.energies[-1]) < 1e-3


def test_observables_match_oracle_and_kats():
    from gato_gb300.grid import Grid3D
    from gato_gb300.observables import kinetic_energy, potential_energy, radial_density, virial_ratio
    og, g = o.Grid3D(48, 10.0), Grid3D(48, 10.0)
    X, Y, Z = og.coords()
    gauss = np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / 2)
    Vh = 0.5 * (X * X + Y * Y + Z * Z)
    d = lambda a: torch.tensor(a, device="cuda")   # noqa: E731
    T = float(kinetic_energy(d(gauss), g))
    assert abs(T - 0.75) < 1e-2                                                  # test_observables.py:14-20
    assert abs(T - o.kinetic_energy(gauss, og)) < 1e-12
    assert abs(float(potential_energy(d(gauss), d(Vh), g)) - o.potential_energy(gauss, Vh, og)) < 1e-12
    assert abs(float(virial_ratio(d(gauss), d(Vh), g)) - 2.0) < 0.05            # test_observables.py:23-36
    psi = np.exp(-np.sqrt(X ** 2 + Y ** 2 + Z ** 2))
    psi = psi / np.sqrt(np.sum(psi * psi) * og.dV)
    r, P = radial_density(d(psi), g, n_bins=80)
    rr, PP = o.radial_density(psi, og, n_bins=80)
    assert np.allclose(r.cpu().numpy(), rr, rtol=0, atol=0)
    assert np.max(np.abs(P.cpu().numpy() - PP)) < 1e-12 * np.max(PP)
    assert abs(float(P.sum()) * float(r[1] - r[0]) - 1.0) < 0.05                # test_observables.py:39-48
    # complex fields: |psi|^2 and the real part of the expectations
    zc = d(psi) * (0.6 + 0.8j)
    assert abs(float(kinetic_energy(zc, g)) - o.kinetic_energy(psi, og)) < 1e-12
    r2, P2 = radial_density(zc, g, n_bins=80)
    assert np.max(np.abs(P2.cpu().numpy() - PP)) < 1e-12 * np.max(PP)
