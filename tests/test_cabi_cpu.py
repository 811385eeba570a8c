"""CPU checks of the boundary and the host logic (no kernel is launched).

* libgato_cuda builds for sm_103a, loads, and exports every entry point
  include/gato.h declares;
* argument validation maps to the reference's exception types before any
  CUDA call;
* host-side helpers (Krylov sizing, pair packing, Adam, E_nn gradient).
"""
import ctypes as C
import os
import re

import pytest
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    src = open(os.path.join(ROOT, "include", "gato.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|long long)\s+(gato_\w+)\s*\(", src, re.M)))


def test_library_exports_every_declared_symbol():
    from gato_gb300 import _lib
    L = _lib.lib()
    syms = header_symbols()
    assert len(syms) >= 35
    for s in syms:
        assert hasattr(L, s), f"{s} declared in gato.h but not exported"
    assert L.gato_version() == 1


def test_python_binding_covers_the_header():
    from gato_gb300 import _lib
    declared = set(header_symbols())
    bound = set(_lib._SIGS) | {"gato_launch_count"}
    assert declared == bound, declared ^ bound


def test_validation_maps_to_reference_exceptions():
    from gato_gb300 import _lib
    L = _lib.lib()
    h = C.c_void_p()
    with pytest.raises(ValueError, match="order"):
        _lib.check(L.gato_op_create(0, 16, 0.25, 3, 0, C.byref(h)))
    with pytest.raises(ValueError, match="boundary"):
        _lib.check(L.gato_op_create(0, 16, 0.25, 4, 7, C.byref(h)))
    with pytest.raises(ValueError):
        _lib.check(L.gato_stencil_apply(0, None, None, None, 1, 8, 8, 8, 1.0, 0, 5, None, 1.0, None))
    with pytest.raises(ValueError):
        _lib.check(L.gato_lanczos(None, None, 10, 4, 1e-10, 1, None, None, None, None, None, None, None))
    with pytest.raises(ValueError, match="rows per thread"):
        _lib.check(L.gato_stencil_tune(3))
    with pytest.raises(ValueError, match="sweeps"):
        _lib.check(L.gato_lanczos_tune(3))
    with pytest.raises(ValueError):
        _lib.boundary_code("mystery")


def test_unsupported_paths_raise_not_implemented():
    from gato_gb300 import _lib
    with pytest.raises(NotImplementedError):
        _lib.check(_lib.GATO_EUNSUPPORTED)
    with pytest.raises(TimeoutError):
        _lib.check(_lib.GATO_ETIMEOUT)


def test_no_cpu_fallback():
    """Without a GPU every operation refuses instead of computing on the host."""
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from gato_gb300.grid import Grid3D, norm_sq
    from gato_gb300.operators import laplacian
    with pytest.raises(RuntimeError, match="CUDA"):
        laplacian(torch.ones(8, 8, 8, dtype=torch.float64), 0.1)
    with pytest.raises(RuntimeError, match="CUDA"):
        norm_sq(torch.ones(8, 8, 8, dtype=torch.float64), Grid3D(8, 1.0))


def test_krylov_dim_and_pair_packing():
    from gato_gb300.scf import pair_fields, precision_dtype
    from gato_gb300.solvers.lanczos import default_krylov_dim
    assert default_krylov_dim(64, 1) == 80 and default_krylov_dim(96, 1) == 120
    assert default_krylov_dim(128, 4) == 160 and default_krylov_dim(160, 4) == 200
    assert default_krylov_dim(40, 4) == 120
    # n(n+1)/2 pairs + the density, two real densities per complex field
    assert [pair_fields(n) for n in (1, 2, 3, 4, 5)] == [1, 2, 4, 6, 8]
    assert precision_dtype("mixed") == torch.float32
    with pytest.raises(ValueError):
        precision_dtype("fp16")


def test_adam_and_geometry_host_logic():
    from gato_gb300.geometry import Nuclei, bond_angle, bond_length, center_of_mass, recenter
    from gato_gb300.geometry_opt import Adam
    from gato_gb300.physics.water import (pp_nuclear_repulsion, pp_nuclear_repulsion_grad,
                                          water_hgh_elements, water_initial_geometry)
    opt = Adam(0.02)
    g = torch.tensor([[0.3, -2.0, 1e-3]], dtype=torch.float64)
    assert torch.allclose(opt.update(g), -0.02 * g / (g.abs() + 1e-8), rtol=1e-12)
    nuc = water_initial_geometry(1.81, 104.5)
    assert float(bond_length(nuc, 0, 1)) == pytest.approx(1.81)
    assert float(bond_angle(nuc, 1, 0, 2)) == pytest.approx(104.5 * 3.141592653589793 / 180)
    assert torch.allclose(center_of_mass(recenter(nuc)), torch.zeros(3, dtype=torch.float64), atol=1e-14)
    el = water_hgh_elements()
    p = nuc.positions.clone().requires_grad_(True)
    E = pp_nuclear_repulsion(Nuclei(p, nuc.charges), el)
    (ga,) = torch.autograd.grad(E, p)
    assert torch.allclose(ga, pp_nuclear_repulsion_grad(nuc, el), rtol=1e-12)


def test_lookup_and_tables():
    from gato_gb300.pseudopotentials import CHLORINE_HGH, OXYGEN_HGH, lookup, total_valence_charge
    from oracle import gato_np as o
    assert lookup("O") is OXYGEN_HGH and lookup("Cl") is CHLORINE_HGH
    for sym in ("H", "Li", "O", "Cl"):
        a, b = lookup(sym), o.lookup(sym)
        assert (a.Z_ion, a.r_loc, a.c) == (b.Z_ion, b.r_loc, b.c)
        assert [(p.ell, p.r, p.h) for p in a.projectors] == [(p.ell, p.r, p.h) for p in b.projectors]
    with pytest.raises(KeyError):
        lookup("Xx")
    assert total_valence_charge((lookup("O"), lookup("H"), lookup("H"))) == 8.0


def test_grid_convergence_variable_projection_fit():
    """The variable-projection fit of benchmarks/grid_convergence.py recovers a known law, stops at a
    bound for a monotone residual, returns None below three points; box studies pick even N."""
    import numpy as np

    from gato_gb300.benchmarks.grid_convergence import box_study, extrapolate
    h = np.array([0.35, 0.3, 0.25, 0.2, 0.15])
    fit = extrapolate(h, -17.3 + 2.0 * h ** 3.5)
    assert abs(fit["y_inf"] + 17.3) < 1e-9 and abs(fit["C"] - 2.0) < 1e-6 and abs(fit["p"] - 3.5) < 1e-6
    assert fit["rms"] < 1e-9 and fit["points"] == 5
    assert extrapolate(h, 1.0 + h ** 0.2)["p"] == 0.5
    assert extrapolate([0.2, 0.1], [1.0, 2.0]) is None
    assert [p.N for p in box_study("hcl", [8.0, 9.0, 10.0], 0.25)] == [32, 36, 40]


def test_bo_gradient_composes_the_adjoint_terms(monkeypatch):
    """The position gradient at fixed orbitals is the sum of the model's adjoint terms (local
    potential, non-local projectors when the model has them, nuclear repulsion) in the adjoint's
    order, returned in the positions' dtype; no energy term is evaluated for it."""
    import torch
    from gato_gb300.grid import Grid3D
    from gato_gb300.physics import _molecule as mol

    calls = []
    monkeypatch.setattr(mol, "to_fields", lambda orb: orb.permute(3, 0, 1, 2))
    monkeypatch.setattr(mol, "_density_fields", lambda f: 2 * (f * f).sum(0))
    monkeypatch.setattr(mol, "_energy_terms", lambda *a, **k: calls.append("energy"))

    class NL:
        def grad(self, fields):
            calls.append("nl")
            return torch.full((2, 3), 0.25, dtype=torch.float64)

    class Model:
        def __init__(self, with_nl):
            self.with_nl = with_nl

        def v_ext_grad(self, nuclei, grid, rho):
            calls.append("v_ext")
            assert nuclei.positions.dtype == torch.float64 and rho.shape == (4, 4, 4)
            return torch.full((2, 3), float(rho.sum()), dtype=torch.float64)

        def nonlocal_op(self, nuclei, grid, dtype):
            return NL() if self.with_nl else None

        def e_nn_grad(self, nuclei):
            calls.append("e_nn")
            return torch.ones((2, 3), dtype=torch.float64)

    orb = torch.ones((4, 4, 4, 1), dtype=torch.float64)
    pos = torch.zeros((2, 3), dtype=torch.float32)
    g = mol.bo_grad_model(Model(True), pos, [1.0, 1.0], orb, Grid3D(4, 2.0))
    assert g.dtype == torch.float32 and torch.allclose(g, torch.full((2, 3), 128.0 + 0.25 + 1.0))
    assert calls == ["v_ext", "nl", "e_nn"]
    calls.clear()
    g = mol.bo_grad_model(Model(False), pos.double(), [1.0, 1.0], orb, Grid3D(4, 2.0))
    assert g.dtype == torch.float64 and torch.allclose(g, torch.full((2, 3), 129.0, dtype=torch.float64))
    assert calls == ["v_ext", "e_nn"]
