"""GPU parity at the shapes the benchmarks run (reference: solvers/poisson.py:47-79, scf.py:66-111,
scf.py:165-286, scf.py:335-444).

* the register FFT engine at N = 96, 128 and 160 (doubled grids 192^3 = 12 x 16, 256^3 = 16 x 16 and
  320^3 = 20 x 16 points per line) against the oracle's exchange_apply and hartree_potential, both
  precisions;
* the block Fock apply of the 128^3 water workload (seeded geometry and orbitals of the benchmark)
  against the oracle in both precisions, and its FP64 energy terms against the oracle's
  decompose_rhf_energy;
* the mixed-precision gate at the benchmark sizes: the 128^3 water SCF against its FP64 continuation,
  and a 160^3 HCl of the 48-system draw, mixed against FP64 energies on identical orbitals.

Tolerances are those of the other parity tests: relative 1e-11 on FP64 fields and 1e-10 Ha on FP64
energies against the oracle; FP32 fields to 2e-5 relative (random inputs: 1e-4), block applies 3e-5;
mixed against FP64 energies within 1e-6 Ha.
"""
import numpy as np
import pytest
import torch

import bench
from oracle import gato_np as o

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    import gato_gb300._lib as L
    L.lib()
    yield
    torch.cuda.synchronize()
    assert L.device_status() == 0, "a bounded device wait expired"


def dev(x, dtype=torch.float64):
    return torch.as_tensor(np.ascontiguousarray(x)).to("cuda", dtype)


def host(t):
    return t.detach().to("cpu", torch.float64).numpy()


def rel_err(got, ref):
    got, ref = np.asarray(got), np.asarray(ref)
    return float(np.max(np.abs(got - ref)) / max(np.max(np.abs(ref)), 1e-300))


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("N", [96, 128, 160])
def test_register_engine_at_benchmark_sizes(dtype, N):
    """Exchange (random orbitals) and Hartree (a smooth density) on the default engine against the
    oracle, M = 2N = 192, 256, 320."""
    from gato_gb300.grid import Grid3D
    from gato_gb300.scf import exchange_apply
    from gato_gb300.solvers.poisson import hartree_potential
    L = 0.25 * N
    og, g = o.Grid3D(N, L), Grid3D(N, L)
    rng = np.random.default_rng(N + 1)
    orbs = rng.standard_normal(og.shape + (2,))
    psi = rng.standard_normal(og.shape)
    ref = o.exchange_apply(psi, orbs, og)
    got = host(exchange_apply(dev(psi, dtype), dev(orbs, dtype), g))
    assert rel_err(got, ref) < (1e-11 if dtype == torch.float64 else 1e-4)
    X, Y, Z = og.coords()
    rho = np.exp(-0.3 * ((X - 0.4) ** 2 + Y ** 2 + (Z + 0.3) ** 2)) * (1.0 + 0.2 * X)
    J = host(hartree_potential(dev(rho, dtype), g))
    assert rel_err(J, o.hartree_potential(rho, og)) < (1e-11 if dtype == torch.float64 else 2e-5)


def _water128(dtype):
    from gato_gb300.geometry import Nuclei
    from gato_gb300.grid import Grid3D
    from gato_gb300.physics.water import water_hgh_elements
    from gato_gb300.pseudopotentials import hgh_local_potential, nonlocal_for
    from gato_gb300.scf import Operator, _density_fields, pair_fields
    from gato_gb300.solvers.poisson import get_plan
    N, h = 128, 0.25
    pos, orbs = bench.synthetic_water(N, h)
    g = Grid3D(N, N * h)
    nuc = Nuclei(torch.tensor(pos), torch.tensor([8.0, 1.0, 1.0], dtype=torch.float64))
    el = water_hgh_elements()
    fields = dev(orbs, dtype)
    V_loc = hgh_local_potential(nuc, el, g, dtype)
    plan = get_plan(N, h, h / 2, dtype, pair_fields(4))
    op = Operator(g, dtype, 4, "dirichlet")
    op.set_potential((V_loc + plan.potential(_density_fields(fields))).contiguous())
    op.set_nonlocal(nonlocal_for(nuc, el, g, dtype))
    op.set_exchange(plan, fields)
    return pos, orbs, op, V_loc


@pytest.fixture(scope="module")
def water128_oracle():
    N, h = 128, 0.25
    pos, orbs = bench.synthetic_water(N, h)
    og = o.Grid3D(N, N * h)
    nuc = o.Nuclei(pos, np.array([8.0, 1.0, 1.0]))
    el = o.water_hgh_elements()
    V_loc = o.hgh_local_potential(nuc, el, og)
    nl = lambda p: o.hgh_nonlocal_apply(p, nuc, el, og)  # noqa: E731
    orb_last = np.moveaxis(orbs, 0, -1)
    V_tot = V_loc + o.hartree_potential(o._density(orb_last), og)
    block = o.fock_apply_block(orbs, V_tot, og, order=4, nl=nl)
    t = o.decompose_rhf_energy(orb_last, V_loc, og, V_nl_apply=nl)
    return block, np.array([t.kinetic, t.v_ext, t.v_nl, t.hartree, t.exchange])


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_water128_block_fock_vs_oracle(dtype, water128_oracle):
    block, terms = water128_oracle
    _, _, op, V_loc = _water128(dtype)
    got = host(op.apply_block())
    assert rel_err(got, block) < (1e-11 if dtype == torch.float64 else 3e-5)
    if dtype == torch.float64:
        e = op.energy_terms(V_loc).cpu().numpy()
        assert np.max(np.abs(e - terms)) < 1e-10, (e, terms)
        assert abs(e.sum() - terms.sum()) < 1e-10


def test_water128_mixed_scf_vs_fp64_continuation():
    """The 128^3 water SCF in mixed precision (stopped at |dE| < 1e-7, its noise floor) against an FP64
    SCF continued from the mixed orbitals: the same fixed point to 1e-6 Ha."""
    from gato_gb300.grid import Grid3D
    from gato_gb300.physics.water import solve_rhf_at_geometry, water_hgh_elements, water_initial_geometry
    from gato_gb300.scf import to_fields
    N, h = 128, 0.25
    g = Grid3D(N, N * h)
    el = water_hgh_elements()
    nuc = water_initial_geometry(1.81, 104.5)
    nuc = type(nuc)(nuc.positions + torch.tensor(np.random.default_rng(11).uniform(-0.05, 0.05, (3, 3))),
                    nuc.charges)
    p32 = solve_rhf_at_geometry(nuc, el, g, precision="mixed", tol=1e-7, max_iters=80)
    assert p32.converged
    p64 = solve_rhf_at_geometry(nuc, el, g, precision="fp64", tol=1e-8, max_iters=6,
                                initial_orbitals=to_fields(p32.orbitals).to(torch.float64).permute(1, 2, 3, 0))
    assert abs(p32.energy - p64.energy) < 1e-6, (p32.energy, p64.energy)


def _hcl160_fields():
    """HCl#17 of the seeded 48-system draw (160^3, h = 0.2015) with four seeded orthonormal orbitals."""
    from gato_gb300.batch import draw_systems
    spec = [s for s in draw_systems(48, seed=0) if s.name == "HCl#17"][0]
    assert spec.N == 160
    pos = spec.nuclei.positions.numpy()
    orbs = bench.synthetic_orbitals(pos, spec.N, spec.h, 4, np.random.default_rng(17))
    return spec, orbs


def test_hcl160_energies_mixed_vs_fp64_identical_orbitals():
    """Energies of the same orbitals at 160^3: the mixed path's reported energy (FP64 terms of the FP32
    orbitals) within 1e-6 Ha of the FP64 path with a 2x margin; the FP32 operator's own energy terms
    (used only early in a mixed SCF) within 1e-5 Ha."""
    from gato_gb300.scf import decompose_rhf_energy, from_fields
    from gato_gb300.pseudopotentials import hgh_local_potential, nonlocal_for
    spec, orbs = _hcl160_fields()
    g = spec.grid
    f64 = dev(orbs)
    f32 = f64.to(torch.float32)
    V64 = hgh_local_potential(spec.nuclei, spec.elements, g, torch.float64)
    V32 = hgh_local_potential(spec.nuclei, spec.elements, g, torch.float32)
    nl64 = nonlocal_for(spec.nuclei, spec.elements, g, torch.float64)
    nl32 = nonlocal_for(spec.nuclei, spec.elements, g, torch.float32)
    E64 = float(decompose_rhf_energy(from_fields(f64), V64, g, order=4, V_nl_apply=nl64).total)
    E_mixed = float(decompose_rhf_energy(from_fields(f32.to(torch.float64)), V64, g, order=4,
                                         V_nl_apply=nl64).total)
    E32 = float(decompose_rhf_energy(from_fields(f32), V32, g, order=4, V_nl_apply=nl32).total)
    assert abs(E_mixed - E64) < 5e-7, (E_mixed, E64)
    assert abs(E32 - E64) < 1e-5, (E32, E64)
