"""CPU oracle: an FP64 NumPy/SciPy restatement of GATO's Fock-operator path.

TEST INFRASTRUCTURE ONLY. This module is the checker, never the product:
only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
and reference legs may import it. The product path (``gato_gb300``) runs on
hand-written CUDA kernels and fails loudly when its library is missing.

Every function restates the reference algorithm it cites (paths relative to
the ezequielgarcia/gato source tree, ``src/gato/...``). The reference is pure
JAX (jax 0.10.0, jaxlib 0.10.0, optax 0.2.8 pinned in ``uv.lock``); JAX is
not installed where this runs, so:

* ``jnp.fft.rfftn/irfftn`` becomes ``scipy.fft.rfftn/irfftn`` (same
  transforms, different roundoff);
* ``jnp.linalg.eigh`` becomes ``numpy.linalg.eigh``;
* ``jax.scipy.special.erf`` becomes ``scipy.special.erf``;
* ``jax.grad`` of the Born-Oppenheimer energy becomes the analytic
  derivative written out below (checked against central differences);
* ``optax.adam`` becomes Adam as published by Kingma & Ba with optax's
  defaults (b1=0.9, b2=0.999, eps=1e-8, eps_root=0).

Parity pinning: the reference ships no golden arrays and cannot be run here,
so this restatement is pinned against the reference's own known-answer tests
(plane-wave eigenvalues, Hermiticity, Gaussian Hartree energy, far field,
linearity, exchange self-reduction, single-orbital energy identity, HO
ladder, helium SCF energy, HGH tail/origin/projector norms, E_nn forces).
Those checks live in ``tests/test_oracle_kats.py``.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field
from typing import Callable, NamedTuple

import numpy as np
import scipy.fft
import scipy.special

_WORKERS = os.cpu_count() or 1


# ---------------------------------------------------------------------------
# grid.py
# ---------------------------------------------------------------------------

@dataclass(frozen=True)
class Grid3D:
    """Cell-centred grid x_i = -L/2 + (i+1/2) h (``grid.py:23-54``)."""

    N: int
    L: float

    @property
    def h(self) -> float:
        return self.L / self.N

    @property
    def shape(self):
        return (self.N, self.N, self.N)

    @property
    def dV(self) -> float:
        return self.h ** 3

    def axis(self) -> np.ndarray:
        return -self.L / 2 + (np.arange(self.N) + 0.5) * self.h

    def coords(self):
        a = self.axis()
        return np.meshgrid(a, a, a, indexing="ij")

    def radial(self, softening: float = 0.0) -> np.ndarray:
        X, Y, Z = self.coords()
        return np.sqrt(X * X + Y * Y + Z * Z + softening * softening)


def integrate(psi, grid):            # grid.py:57-59
    return np.sum(psi) * grid.dV


def inner_product(phi, psi, grid):   # grid.py:62-64
    return np.sum(np.conj(phi) * psi) * grid.dV


def norm_sq(psi, grid):              # grid.py:67-69
    return np.sum(np.abs(psi) ** 2) * grid.dV


def normalize(psi, grid):            # grid.py:72-73
    return psi / np.sqrt(norm_sq(psi, grid))


# ---------------------------------------------------------------------------
# operators.py
# ---------------------------------------------------------------------------

_C4_1 = 16.0 / 12.0      # operators.py:34
_C4_2 = -1.0 / 12.0      # operators.py:35
_C4_0 = -30.0 / 12.0     # operators.py:36


def laplacian(psi, h, boundary="dirichlet", order=2):
    """7-point / 13-point Laplacian (``operators.py:40-119``)."""
    if order == 2:
        return _laplacian_order2(psi, h, boundary)
    if order == 4:
        return _laplacian_order4(psi, h, boundary)
    raise ValueError(f"Unknown order {order!r}; expected 2 or 4.")


def _laplacian_order2(psi, h, boundary):
    """``operators.py:67-84``: periodic via roll, Dirichlet via zero pad."""
    if boundary == "periodic":
        acc = -6.0 * psi
        for ax in range(3):
            acc = acc + np.roll(psi, 1, axis=ax) + np.roll(psi, -1, axis=ax)
    elif boundary == "dirichlet":
        p = np.pad(psi, 1)
        acc = (p[2:, 1:-1, 1:-1] + p[:-2, 1:-1, 1:-1]
               + p[1:-1, 2:, 1:-1] + p[1:-1, :-2, 1:-1]
               + p[1:-1, 1:-1, 2:] + p[1:-1, 1:-1, :-2]
               + -6.0 * p[1:-1, 1:-1, 1:-1])
    else:
        raise ValueError(f"Unknown boundary {boundary!r}; expected 'dirichlet' or 'periodic'.")
    return acc / (h * h)


def _laplacian_order4(psi, h, boundary):
    """``operators.py:87-119``: centre 3*(-30/12), +-1: 16/12, +-2: -1/12."""
    center = 3.0 * _C4_0
    if boundary == "periodic":
        acc = center * psi
        for ax in range(3):
            acc = (acc + _C4_1 * (np.roll(psi, 1, axis=ax) + np.roll(psi, -1, axis=ax))
                   + _C4_2 * (np.roll(psi, 2, axis=ax) + np.roll(psi, -2, axis=ax)))
    elif boundary == "dirichlet":
        p = np.pad(psi, 2)
        c = slice(2, -2)
        acc = (center * p[c, c, c]
               + _C4_1 * (p[3:-1, c, c] + p[1:-3, c, c])
               + _C4_2 * (p[4:, c, c] + p[:-4, c, c])
               + _C4_1 * (p[c, 3:-1, c] + p[c, 1:-3, c])
               + _C4_2 * (p[c, 4:, c] + p[c, :-4, c])
               + _C4_1 * (p[c, c, 3:-1] + p[c, c, 1:-3])
               + _C4_2 * (p[c, c, 4:] + p[c, c, :-4]))
    else:
        raise ValueError(f"Unknown boundary {boundary!r}; expected 'dirichlet' or 'periodic'.")
    return acc / (h * h)


def kinetic(psi, h, boundary="dirichlet", order=2):   # operators.py:122-130
    return -0.5 * laplacian(psi, h, boundary, order)


# ---------------------------------------------------------------------------
# hamiltonian.py
# ---------------------------------------------------------------------------

@dataclass(frozen=True)
class Hamiltonian:
    """H = T + V (``hamiltonian.py:18-35``)."""

    grid: Grid3D
    V: np.ndarray
    boundary: str = "dirichlet"
    order: int = 2

    def apply(self, psi):
        return kinetic(psi, self.grid.h, self.boundary, self.order) + self.V * psi

    def expectation(self, psi):
        return inner_product(psi, self.apply(psi), self.grid).real

    def rayleigh(self, psi):
        return self.expectation(psi) / norm_sq(psi, self.grid).real


# ---------------------------------------------------------------------------
# geometry.py / potentials.py
# ---------------------------------------------------------------------------

class Nuclei(NamedTuple):
    """``geometry.py:20-28``."""

    positions: np.ndarray   # (K, 3)
    charges: np.ndarray     # (K,)

    @property
    def n(self) -> int:
        return int(self.charges.shape[0])


def diatomic_along_z(R, Z1, Z2=None):      # geometry.py:31-45
    if Z2 is None:
        Z2 = Z1
    return Nuclei(np.array([[0.0, 0.0, -R / 2], [0.0, 0.0, R / 2]]), np.asarray([Z1, Z2], float))


def bond_length(nuclei, i, j):             # geometry.py:48-50
    return float(np.linalg.norm(nuclei.positions[i] - nuclei.positions[j]))


def bond_angle(nuclei, i, j, k):           # geometry.py:53-58
    a = nuclei.positions[i] - nuclei.positions[j]
    b = nuclei.positions[k] - nuclei.positions[j]
    c = np.dot(a, b) / (np.linalg.norm(a) * np.linalg.norm(b))
    return float(np.arccos(np.clip(c, -1.0, 1.0)))


def nuclear_repulsion(nuclei):             # geometry.py:61-75
    K = nuclei.n
    if K < 2:
        return 0.0
    i, j = np.triu_indices(K, k=1)
    r = np.linalg.norm(nuclei.positions[i] - nuclei.positions[j], axis=-1)
    return float(np.sum(nuclei.charges[i] * nuclei.charges[j] / r))


def nuclear_repulsion_grad(nuclei):
    """d E_nn / d R, the analytic form of ``jax.grad(nuclear_repulsion)``."""
    K = nuclei.n
    g = np.zeros((K, 3))
    for a in range(K):
        for b in range(K):
            if a == b:
                continue
            d = nuclei.positions[a] - nuclei.positions[b]
            r = np.linalg.norm(d)
            g[a] += -nuclei.charges[a] * nuclei.charges[b] * d / r ** 3
    return g


def center_of_mass(nuclei):                # geometry.py:78-83
    return (nuclei.charges[:, None] * nuclei.positions).sum(axis=0) / nuclei.charges.sum()


def recenter(nuclei):                      # geometry.py:86-91
    return Nuclei(nuclei.positions - center_of_mass(nuclei), nuclei.charges)


def softened_coulomb(grid, Z=1.0, epsilon=None, center=(0.0, 0.0, 0.0)):   # potentials.py:16-36
    if epsilon is None:
        epsilon = grid.h / 2
    X, Y, Zc = grid.coords()
    x0, y0, z0 = center
    r2 = (X - x0) ** 2 + (Y - y0) ** 2 + (Zc - z0) ** 2
    return -Z / np.sqrt(r2 + epsilon * epsilon)


def multi_center_softened_coulomb(nuclei, grid, epsilon=None):              # potentials.py:39-61
    if epsilon is None:
        epsilon = grid.h / 2
    X, Y, Zc = grid.coords()
    V = np.zeros(grid.shape)
    for R, Zk in zip(nuclei.positions, nuclei.charges):
        r2 = (X - R[0]) ** 2 + (Y - R[1]) ** 2 + (Zc - R[2]) ** 2
        V = V + (-Zk / np.sqrt(r2 + epsilon * epsilon))
    return V


def multi_center_softened_coulomb_grad(nuclei, grid, rho, epsilon=None):
    """d/dR_k of int rho V_ext dV for V_ext = multi_center_softened_coulomb: the force term
    physics/h2.py:109-135 takes with jax.grad; analytic: -Z_k (r - R_k) / (|r - R_k|^2 + eps^2)^{3/2}."""
    if epsilon is None:
        epsilon = grid.h / 2
    X, Y, Zc = grid.coords()
    g = np.zeros((len(nuclei.charges), 3))
    for k, (R, Zk) in enumerate(zip(nuclei.positions, nuclei.charges)):
        d = (X - R[0], Y - R[1], Zc - R[2])
        w = -Zk * rho / (d[0] ** 2 + d[1] ** 2 + d[2] ** 2 + epsilon * epsilon) ** 1.5
        for c in range(3):
            g[k, c] = np.sum(w * d[c]) * grid.dV
    return g


def harmonic_oscillator(grid, omega=1.0):  # potentials.py:64-69 (test fixture)
    X, Y, Z = grid.coords()
    return 0.5 * omega * omega * (X * X + Y * Y + Z * Z)


def constant(grid, v0=0.0):                # potentials.py:72-76 (test fixture)
    return np.full(grid.shape, float(v0))


# ---------------------------------------------------------------------------
# pseudopotentials.py
# ---------------------------------------------------------------------------

@dataclass(frozen=True)
class HGHProjector:
    ell: int
    r: float
    h: tuple

    @property
    def n(self) -> int:
        return len(self.h)


@dataclass(frozen=True)
class HGHParams:
    symbol: str
    Z_ion: float
    r_loc: float
    c: tuple
    projectors: tuple = ()


# Hartwigsen-Goedecker-Hutter 1998 table I (LDA), as tabulated in
# pseudopotentials.py:122-185. The values are physical constants of the
# published pseudopotentials and must be identical for parity.
HYDROGEN_HGH = HGHParams("H", 1.0, 0.2, (-4.0663326, 0.6778322, 0.0, 0.0), ())
OXYGEN_HGH = HGHParams("O", 6.0, 0.24762086, (-16.5803180, 2.39570952, 0.0, 0.0),
                       (HGHProjector(0, 0.22178614, ((18.26691718,),)),))
LITHIUM_HGH = HGHParams("Li", 1.0, 0.78755305, (-1.89261247, 0.28605968, 0.0, 0.0),
                        (HGHProjector(0, 0.66637518, ((1.85881111,),)),
                         HGHProjector(1, 1.07930561, ((-0.00589504,),))))
CHLORINE_HGH = HGHParams("Cl", 7.0, 0.41, (-6.86475431, 0.0, 0.0, 0.0),
                         (HGHProjector(0, 0.33820832, ((9.06223968, -1.96193036),
                                                       (-1.96193036, 5.06568240))),
                          HGHProjector(1, 0.37613709, ((4.46587640,),))))
HGH_TABLE = {"H": HYDROGEN_HGH, "Li": LITHIUM_HGH, "O": OXYGEN_HGH, "Cl": CHLORINE_HGH}


def lookup(symbol):                        # pseudopotentials.py:188-194
    if symbol not in HGH_TABLE:
        raise KeyError(f"No HGH parameters for {symbol!r}.")
    return HGH_TABLE[symbol]


def total_valence_charge(elements):        # pseudopotentials.py:256-258
    return float(sum(p.Z_ion for p in elements))


def _grid_pts(grid):
    X, Y, Z = grid.coords()
    return np.stack([X, Y, Z], axis=-1)


def _hgh_local_one_center(grid_pts, R, params):   # pseudopotentials.py:201-227
    diff = grid_pts - R
    r2 = np.sum(diff * diff, axis=-1)
    r = np.sqrt(r2 + 1e-30)
    rho = r / params.r_loc
    erf_term = -params.Z_ion * scipy.special.erf(r / (math.sqrt(2.0) * params.r_loc)) / r
    c1, c2, c3, c4 = params.c
    rho2 = rho * rho
    poly = c1 + c2 * rho2 + c3 * rho2 * rho2 + c4 * rho2 * rho2 * rho2
    return erf_term + np.exp(-0.5 * rho2) * poly


def hgh_local_potential(nuclei, elements, grid):  # pseudopotentials.py:230-253
    if len(elements) != nuclei.n:
        raise ValueError(f"HGH parameter list length {len(elements)} != number of nuclei {nuclei.n}")
    pts = _grid_pts(grid)
    V = np.zeros(grid.shape)
    for k, params in enumerate(elements):
        V = V + _hgh_local_one_center(pts, nuclei.positions[k], params)
    return V


def _projector_radial(r, ell, i_idx, r_ell):       # pseudopotentials.py:265-277
    n = ell + (4 * i_idx - 1) / 2.0
    norm = math.sqrt(2.0) / (r_ell ** n * math.sqrt(math.gamma(n)))
    power = ell + 2 * (i_idx - 1)
    return norm * (r ** power) * np.exp(-(r * r) / (2.0 * r_ell * r_ell))


def _angular_factor(ell, m, hat):                   # pseudopotentials.py:280-309
    if ell == 0 and m == 0:
        return np.full(hat.shape[:-1], 1.0 / math.sqrt(4.0 * math.pi))
    if ell == 1:
        c = math.sqrt(3.0 / (4.0 * math.pi))
        return c * hat[..., {-1: 1, 0: 2, 1: 0}[m]]
    if ell == 2:
        x, y, z = hat[..., 0], hat[..., 1], hat[..., 2]
        if m == -2:
            return math.sqrt(15.0 / (4.0 * math.pi)) * x * y
        if m == -1:
            return math.sqrt(15.0 / (4.0 * math.pi)) * y * z
        if m == 0:
            return 0.25 * math.sqrt(5.0 / math.pi) * (3.0 * z * z - 1.0)
        if m == 1:
            return math.sqrt(15.0 / (4.0 * math.pi)) * x * z
        if m == 2:
            return 0.25 * math.sqrt(15.0 / math.pi) * (x * x - y * y)
    raise NotImplementedError(f"Real Y_{{{ell},{m}}} not implemented (need l <= 2).")


def _projector_field(grid_pts, R, ell, m, i_idx, r_ell):   # pseudopotentials.py:312-327
    diff = grid_pts - R
    r2 = np.sum(diff * diff, axis=-1)
    r = np.sqrt(r2 + 1e-30)
    radial = _projector_radial(r, ell, i_idx, r_ell)
    hat = diff / r[..., None]
    return radial * _angular_factor(ell, m, hat)


def _projector_list(nuclei, elements):
    """Flatten (atom, l, m) channels; each holds its n radial projectors and h."""
    out = []
    for k, params in enumerate(elements):
        for proj in params.projectors:
            for m in range(-proj.ell, proj.ell + 1):
                out.append((k, proj.ell, m, proj.r, np.asarray(proj.h, float)))
    return out


def hgh_nonlocal_apply(psi, nuclei, elements, grid):         # pseudopotentials.py:330-383
    pts = _grid_pts(grid)
    out = np.zeros_like(psi)
    for k, ell, m, r_ell, h in _projector_list(nuclei, elements):
        ps = [_projector_field(pts, nuclei.positions[k], ell, m, i + 1, r_ell) for i in range(h.shape[0])]
        ov = np.array([inner_product(p, psi, grid).real for p in ps])
        coeffs = h @ ov
        for i in range(h.shape[0]):
            out = out + coeffs[i] * ps[i]
    return out


def hgh_apply(psi, nuclei, elements, grid, V_local=None):    # pseudopotentials.py:390-405
    if V_local is None:
        V_local = hgh_local_potential(nuclei, elements, grid)
    return V_local * psi + hgh_nonlocal_apply(psi, nuclei, elements, grid)


# ---- analytic position derivatives (the oracle's restatement of jax.grad) --

def _hgh_local_radial_deriv(r, params):
    """dV_loc/dr for one centre, differentiating pseudopotentials.py:214-227."""
    a = math.sqrt(2.0) * params.r_loc
    u = r / a
    erf_u = scipy.special.erf(u)
    derf = 2.0 / math.sqrt(math.pi) * np.exp(-u * u) / a
    d_erf_term = -params.Z_ion * (derf / r - erf_u / (r * r))
    rho2 = (r / params.r_loc) ** 2
    c1, c2, c3, c4 = params.c
    poly = c1 + c2 * rho2 + c3 * rho2 ** 2 + c4 * rho2 ** 3
    dpoly = c2 + 2 * c3 * rho2 + 3 * c4 * rho2 ** 2          # dP/d(rho2)
    drho2 = 2.0 * r / params.r_loc ** 2
    d_poly_term = np.exp(-0.5 * rho2) * (-0.5 * poly + dpoly) * drho2
    return d_erf_term + d_poly_term


def hgh_local_force_density(nuclei, elements, grid, rho):
    """d/dR_k of ∫ rho V_loc dV, shape (K, 3)."""
    pts = _grid_pts(grid)
    g = np.zeros((nuclei.n, 3))
    for k, params in enumerate(elements):
        diff = pts - nuclei.positions[k]
        r = np.sqrt(np.sum(diff * diff, axis=-1) + 1e-30)
        dV = _hgh_local_radial_deriv(r, params)
        # dV/dR = dV/dr * dr/dR = dV/dr * (-(x - R)/r)
        w = rho * dV / r
        g[k] = -np.einsum("xyz,xyzc->c", w, diff) * grid.dV
    return g


def _solid_harmonic(ell, m, d):
    """r^l Y_lm(r_hat) as a polynomial in d (drops the 1e-30 floor)."""
    x, y, z = d[..., 0], d[..., 1], d[..., 2]
    if ell == 0:
        return np.full(d.shape[:-1], 1.0 / math.sqrt(4.0 * math.pi)), np.zeros(d.shape)
    if ell == 1:
        c = math.sqrt(3.0 / (4.0 * math.pi))
        ax = {-1: 1, 0: 2, 1: 0}[m]
        g = np.zeros(d.shape)
        g[..., ax] = c
        return c * d[..., ax], g
    raise NotImplementedError("projector gradients implemented for l <= 1 (H, Li, O, Cl)")


def _projector_field_and_grad(grid_pts, R, ell, m, i_idx, r_ell):
    """p(d) = norm r^{2(i-1)} S_lm(d) exp(-r^2/2r_l^2) and its d-gradient."""
    diff = grid_pts - R
    r2 = np.sum(diff * diff, axis=-1) + 1e-30
    n = ell + (4 * i_idx - 1) / 2.0
    norm = math.sqrt(2.0) / (r_ell ** n * math.sqrt(math.gamma(n)))
    q = i_idx - 1
    g = np.exp(-r2 / (2.0 * r_ell * r_ell))
    S, dS = _solid_harmonic(ell, m, diff)
    rq = r2 ** q
    f = norm * rq * S * g
    drq = (2 * q * r2 ** (q - 1))[..., None] * diff if q > 0 else 0.0
    grad = norm * (drq * (S * g)[..., None] + (rq * g)[..., None] * dS
                   - (rq * S * g)[..., None] * diff / (r_ell * r_ell))
    return f, grad


def hgh_nonlocal_energy_grad(nuclei, elements, grid, orbitals):
    """d/dR of 2 Σ_i <φ_i|V_nl|φ_i>, shape (K, 3); orbitals (n, N, N, N)."""
    pts = _grid_pts(grid)
    g = np.zeros((nuclei.n, 3))
    for k, ell, m, r_ell, h in _projector_list(nuclei, elements):
        fs, grads = zip(*[_projector_field_and_grad(pts, nuclei.positions[k], ell, m, i + 1, r_ell)
                          for i in range(h.shape[0])])
        for phi in orbitals:
            ov = np.array([np.sum(f * phi) * grid.dV for f in fs])
            # d<p|φ>/dR = -∫ grad_d p φ
            dov = np.array([-np.einsum("xyzc,xyz->c", gr, phi) * grid.dV for gr in grads])
            # d(ov^T h ov) = 2 ov^T h dov
            g[k] += 2.0 * 2.0 * (h @ ov) @ dov
    return g


# ---------------------------------------------------------------------------
# solvers/poisson.py
# ---------------------------------------------------------------------------

def _coulomb_kernel(N, h, epsilon):        # poisson.py:29-44
    M = 2 * N
    idx = np.arange(M)
    disp = np.where(idx < N, idx * h, (idx - M) * h)
    X = disp[:, None, None]
    Y = disp[None, :, None]
    Z = disp[None, None, :]
    return 1.0 / np.sqrt(X * X + Y * Y + Z * Z + epsilon * epsilon)


_GHAT_CACHE: dict = {}


def _kernel_hat(N, h, epsilon):
    """rfftn(G). The reference rebuilds it every call; caching is value-neutral."""
    key = (N, float(h), float(epsilon))
    if key not in _GHAT_CACHE:
        if len(_GHAT_CACHE) > 4:
            _GHAT_CACHE.clear()
        _GHAT_CACHE[key] = scipy.fft.rfftn(_coulomb_kernel(N, h, epsilon), workers=_WORKERS)
    return _GHAT_CACHE[key]


def hartree_potential(rho, grid, epsilon=None):   # poisson.py:47-79
    if epsilon is None:
        epsilon = grid.h / 2
    N = grid.N
    M = 2 * N
    pad = np.zeros((M, M, M))
    pad[:N, :N, :N] = rho
    J = scipy.fft.irfftn(scipy.fft.rfftn(pad, workers=_WORKERS) * _kernel_hat(N, grid.h, epsilon),
                         s=(M, M, M), workers=_WORKERS)
    return J[:N, :N, :N] * grid.dV


def hartree_energy(rho, grid, epsilon=None):      # poisson.py:82-92
    J = hartree_potential(rho, grid, epsilon)
    return 0.5 * integrate(rho * J, grid)


# ---------------------------------------------------------------------------
# solvers/lanczos.py
# ---------------------------------------------------------------------------

@dataclass
class LanczosResult:
    eigenvalues: np.ndarray   # (K,)
    eigenstates: np.ndarray   # (N, N, N, K)
    n_iters: int
    converged: bool
    alphas: np.ndarray = None
    betas: np.ndarray = None


def default_krylov_dim(N, n_eigenstates=1):      # lanczos.py:49-107
    return max(24 * n_eigenstates + 24, (5 * N) // 4)


def lanczos(H, psi0, n_iters=80, n_eigenstates=4, tol=1e-10):   # lanczos.py:110-206
    """Single-vector Lanczos with MGS full reorthogonalisation."""
    grid = H.grid
    shape = psi0.shape
    v0 = psi0 / np.sqrt(norm_sq(psi0, grid).real)
    Vb = np.zeros((n_iters + 1,) + shape)
    Vb[0] = v0
    alphas = np.zeros(n_iters)
    betas = np.zeros(n_iters)
    for j in range(n_iters):
        v_j = Vb[j]
        w = H.apply(v_j)
        if j > 0:
            w = w - betas[j - 1] * Vb[j - 1]
        alpha = inner_product(v_j, w, grid).real
        alphas[j] = alpha
        w = w - alpha * v_j
        for k in range(j + 1):                       # lanczos.py:155-159 (MGS)
            coeff = inner_product(Vb[k], w, grid).real
            w = w - coeff * Vb[k]
        beta = math.sqrt(norm_sq(w, grid).real)
        betas[j] = beta
        Vb[j + 1] = w / beta if beta > 0 else np.zeros_like(w)
    T = np.diag(alphas)
    if n_iters >= 2:
        off = betas[: n_iters - 1]
        T = T + np.diag(off, 1) + np.diag(off, -1)
    evals, evecs = np.linalg.eigh(T)
    # LAPACK leaves each eigenvector's sign arbitrary (the reference inherits its
    # platform's choice); fix it as the device solver does: the component of
    # largest magnitude is positive. Energies and densities do not depend on
    # it; the SCF seed sum(orbitals) does.
    idx = np.argmax(np.abs(evecs), axis=0)
    evecs = evecs * np.where(evecs[idx, np.arange(evecs.shape[1])] < 0, -1.0, 1.0)
    K = min(n_eigenstates, n_iters)
    V_stack = Vb[:n_iters].reshape(n_iters, -1)
    psi_states = (evecs[:, :K].T @ V_stack).reshape(K, *shape)
    converged = bool(np.any(betas[: max(n_iters - 1, 1)] < tol))
    return LanczosResult(evals[:K], np.transpose(psi_states, (1, 2, 3, 0)), int(n_iters), converged,
                         alphas, betas)


def imaginary_time(H, psi0, dt=None, n_steps=2000):
    """Euler imaginary-time propagation (``solvers/imag_time.py:29-65``), for KATs.

    Returns (psi, final Rayleigh quotient)."""
    grid = H.grid
    if dt is None:
        dt = grid.h ** 2 / 10.0
    psi = psi0 / np.sqrt(norm_sq(psi0, grid))
    for _ in range(n_steps):
        psi_new = psi - dt * H.apply(psi)
        psi = psi_new / np.sqrt(norm_sq(psi_new, grid))
    return psi, float(H.rayleigh(psi))


def imaginary_time_logged(H, psi0, dt=None, n_steps=2000, log_every=50):
    """solvers/imag_time.py:29-65 with its log: (psi, steps, Rayleigh quotients)."""
    grid = H.grid
    if dt is None:
        dt = grid.h ** 2 / 10.0
    psi = psi0 / np.sqrt(norm_sq(psi0, grid))
    steps, energies = [], []
    for i in range(n_steps):
        psi_new = psi - dt * H.apply(psi)
        psi = psi_new / np.sqrt(norm_sq(psi_new, grid))
        if i % log_every == 0 or i == n_steps - 1:
            steps.append(i)
            energies.append(float(H.rayleigh(psi)))
    return psi, steps, energies


# ---------------------------------------------------------------------------
# observables.py
# ---------------------------------------------------------------------------

def kinetic_energy(psi, grid, boundary="dirichlet", order=2):     # observables.py:16-21
    return inner_product(psi, kinetic(psi, grid.h, boundary, order), grid).real / norm_sq(psi, grid).real


def potential_energy(psi, V, grid):                               # observables.py:24-28
    return inner_product(psi, V * psi, grid).real / norm_sq(psi, grid).real


def virial_ratio(psi, V, grid, boundary="dirichlet", order=2):    # observables.py:31-44
    return 2 * kinetic_energy(psi, grid, boundary, order) / abs(potential_energy(psi, V, grid))


def radial_density(psi, grid, n_bins=100, r_max=None):            # observables.py:47-59
    r = grid.radial().reshape(-1)
    density = (np.abs(psi) ** 2 * grid.dV).reshape(-1)
    if r_max is None:
        r_max = float(grid.L / 2)
    bins = np.linspace(0.0, r_max, n_bins + 1)
    centers = 0.5 * (bins[1:] + bins[:-1])
    widths = bins[1:] - bins[:-1]
    hist, _ = np.histogram(r, bins=bins, weights=density)
    return centers, hist / widths


# ---------------------------------------------------------------------------
# scf.py
# ---------------------------------------------------------------------------

def _density(orbitals):                    # scf.py:61-63, orbitals (N,N,N,n)
    return 2.0 * np.sum(np.abs(orbitals) ** 2, axis=-1)


def exchange_apply(psi, orbitals, grid, epsilon=None):     # scf.py:66-85
    out = np.zeros_like(psi)
    for j in range(orbitals.shape[-1]):
        phi_j = orbitals[..., j]
        out = out + phi_j * hartree_potential(np.conj(phi_j) * psi, grid, epsilon=epsilon)
    return out


@dataclass(frozen=True)
class RHFFock:
    """``scf.py:114-158``."""

    grid: Grid3D
    V_ext: np.ndarray
    orbitals: np.ndarray
    V_H: np.ndarray = None
    boundary: str = "dirichlet"
    order: int = 4
    epsilon: float = None
    V_nl_apply: Callable = None

    def density(self):
        return _density(self.orbitals)

    def hartree(self):
        if self.V_H is not None:
            return self.V_H
        return hartree_potential(self.density(), self.grid, epsilon=self.epsilon)

    def apply(self, psi):                  # _fock_apply_kernel, scf.py:88-111
        eps = self.grid.h / 2 if self.epsilon is None else self.epsilon
        h_psi = kinetic(psi, self.grid.h, self.boundary, self.order) + self.V_ext * psi
        if self.V_nl_apply is not None:
            h_psi = h_psi + self.V_nl_apply(psi)
        return h_psi + self.hartree() * psi - exchange_apply(psi, self.orbitals, self.grid, eps)


@dataclass(frozen=True)
class RHFEnergyTerms:
    """``scf.py:165-191``."""

    kinetic: float
    v_ext: float
    v_nl: float
    hartree: float
    exchange: float

    @property
    def one_body(self):
        return self.kinetic + self.v_ext + self.v_nl

    @property
    def total(self):
        return self.kinetic + self.v_ext + self.v_nl + self.hartree + self.exchange


def decompose_rhf_energy(orbitals, V_ext, grid, *, boundary="dirichlet", order=4,
                         epsilon=None, V_nl_apply=None):           # scf.py:194-265
    if epsilon is None:
        epsilon = grid.h / 2
    n_orb = orbitals.shape[-1]
    T = V_ext_exp = V_nl_exp = 0.0
    for i in range(n_orb):
        phi = orbitals[..., i]
        T += inner_product(phi, kinetic(phi, grid.h, boundary, order), grid).real
        V_ext_exp += inner_product(phi, V_ext * phi, grid).real
        if V_nl_apply is not None:
            V_nl_exp += inner_product(phi, V_nl_apply(phi), grid).real
    E_H = hartree_energy(_density(orbitals), grid, epsilon=epsilon)
    E_x = 0.0
    for i in range(n_orb):
        phi = orbitals[..., i]
        E_x -= inner_product(phi, exchange_apply(phi, orbitals, grid, epsilon), grid).real
    return RHFEnergyTerms(float(2 * T), float(2 * V_ext_exp), float(2 * V_nl_exp), float(E_H), float(E_x))


def rhf_energy(orbitals, V_ext, grid, boundary="dirichlet", order=4, epsilon=None, V_nl_apply=None):
    return decompose_rhf_energy(orbitals, V_ext, grid, boundary=boundary, order=order,
                                epsilon=epsilon, V_nl_apply=V_nl_apply).total   # scf.py:268-286


def default_initial_guess(grid):
    """Starter vector of ``_default_initial_orbitals`` (``scf.py:310-320``)."""
    X, Y, Z = grid.coords()
    r = np.sqrt(X * X + Y * Y + Z * Z + 1e-6)
    return (np.exp(-4.0 * r) + np.exp(-r)) * (1.0 + 0.1 * (X + Y + Z) + 0.02 * (X * Y + Y * Z + X * Z))


def _default_initial_orbitals(V_ext, grid, n_occ, boundary, order, lanczos_iters):   # scf.py:289-322
    H_core = Hamiltonian(grid, V_ext, boundary, order)
    return lanczos(H_core, default_initial_guess(grid), n_iters=lanczos_iters, n_eigenstates=n_occ).eigenstates


@dataclass
class SCFResult:
    orbitals: np.ndarray
    energy: float
    orbital_energies: np.ndarray
    n_iters: int
    converged: bool
    energy_history: list = field(default_factory=list)


def scf_rhf(V_ext, grid, n_occ, *, initial_orbitals=None, max_iters=50, tol=1e-6, mixing=1.0,
            boundary="dirichlet", order=4, lanczos_iters=None, epsilon=None, V_nl_apply=None):
    """``scf.py:335-444``: Lanczos on the Fock built from the mixed density."""
    if lanczos_iters is None:
        lanczos_iters = default_krylov_dim(grid.N, n_occ)
    if initial_orbitals is None:
        orbitals = _default_initial_orbitals(V_ext, grid, n_occ, boundary, order, lanczos_iters)
    else:
        orbitals = initial_orbitals
    history = []
    rho = _density(orbitals)
    E_prev = float("inf")
    E = float("inf")
    orbital_energies = np.zeros(n_occ)
    converged = False
    it = 0
    for it in range(1, max_iters + 1):
        V_H = hartree_potential(rho, grid, epsilon=epsilon)
        fock = RHFFock(grid, V_ext, orbitals, V_H, boundary, order, epsilon, V_nl_apply)
        seed = np.sum(orbitals, axis=-1)
        res = lanczos(fock, seed, n_iters=lanczos_iters, n_eigenstates=n_occ)
        new_orbitals = res.eigenstates
        orbital_energies = res.eigenvalues
        rho = mixing * _density(new_orbitals) + (1.0 - mixing) * rho
        orbitals = new_orbitals
        E = float(rhf_energy(orbitals, V_ext, grid, boundary, order, epsilon=epsilon, V_nl_apply=V_nl_apply))
        history.append(E)
        if abs(E - E_prev) < tol:
            converged = True
            break
        E_prev = E
    return SCFResult(orbitals, E, orbital_energies, it, converged, history)


# ---------------------------------------------------------------------------
# Block Fock apply (the benchmark unit): F φ_i for every occupied orbital.
# Algebraically the same as applying scf.py:88-111 to each φ_i.
# ---------------------------------------------------------------------------

def fock_apply_block(orbitals_first, V_tot, grid, order=4, epsilon=None, nl=None):
    """F φ_i for i < n with V_tot = V_ext + V_H; orbitals_first is (n, N, N, N).

    Uses the pair symmetry J[φ_iφ_j] = J[φ_jφ_i], so n(n+1)/2 Poisson solves.
    ``nl`` is an optional callable ψ -> V_nl ψ.
    """
    if epsilon is None:
        epsilon = grid.h / 2
    n = orbitals_first.shape[0]
    out = np.empty_like(orbitals_first)
    for i in range(n):
        out[i] = kinetic(orbitals_first[i], grid.h, "dirichlet", order) + V_tot * orbitals_first[i]
        if nl is not None:
            out[i] += nl(orbitals_first[i])
    for i in range(n):
        for j in range(i, n):
            Jij = hartree_potential(orbitals_first[i] * orbitals_first[j], grid, epsilon)
            out[i] -= orbitals_first[j] * Jij
            if j != i:
                out[j] -= orbitals_first[i] * Jij
    return out


# ---------------------------------------------------------------------------
# geometry_opt.py (Adam restated) and physics/water.py
# ---------------------------------------------------------------------------

class Adam:
    """Kingma & Ba (2015) with optax.adam defaults (geometry_opt.py:61-71)."""

    def __init__(self, lr, b1=0.9, b2=0.999, eps=1e-8):
        self.lr, self.b1, self.b2, self.eps = lr, b1, b2, eps
        self.mu = self.nu = None
        self.count = 0

    def update(self, g):
        if self.mu is None:
            self.mu = np.zeros_like(g)
            self.nu = np.zeros_like(g)
        self.count += 1
        self.mu = self.b1 * self.mu + (1 - self.b1) * g
        self.nu = self.b2 * self.nu + (1 - self.b2) * g * g
        mu_hat = self.mu / (1 - self.b1 ** self.count)
        nu_hat = self.nu / (1 - self.b2 ** self.count)
        return -self.lr * mu_hat / (np.sqrt(nu_hat) + self.eps)


def water_initial_geometry(R_OH=1.85, angle_deg=100.0):     # water.py:66-82
    half = np.deg2rad(angle_deg) / 2.0
    h1 = [R_OH * np.sin(half), 0.0, R_OH * np.cos(half)]
    h2 = [-R_OH * np.sin(half), 0.0, R_OH * np.cos(half)]
    return Nuclei(np.array([[0.0, 0.0, 0.0], h1, h2]), np.array([8.0, 1.0, 1.0]))


def water_hgh_elements():                                   # water.py:85-87
    return (lookup("O"), lookup("H"), lookup("H"))


def pp_nuclear_repulsion(nuclei, elements):                 # water.py:100-110
    return nuclear_repulsion(Nuclei(nuclei.positions, np.asarray([p.Z_ion for p in elements], float)))


def pp_nuclear_repulsion_grad(nuclei, elements):
    return nuclear_repulsion_grad(Nuclei(nuclei.positions, np.asarray([p.Z_ion for p in elements], float)))


def bo_energy(positions, charges, orbitals, elements, grid, order=4):   # water.py:181-215
    nuclei = Nuclei(np.asarray(positions, float), np.asarray(charges, float))
    V_local = hgh_local_potential(nuclei, elements, grid)
    terms = decompose_rhf_energy(orbitals, V_local, grid, boundary="dirichlet", order=order, epsilon=None,
                                 V_nl_apply=lambda p: hgh_nonlocal_apply(p, nuclei, elements, grid))
    return terms.total + pp_nuclear_repulsion(nuclei, elements)


def bo_energy_position_part(positions, charges, orbitals, elements, grid):
    """The R-dependent part of bo_energy (V_loc, V_nl, E_nn); T, E_H, E_x are R-independent."""
    nuclei = Nuclei(np.asarray(positions, float), np.asarray(charges, float))
    rho = _density(orbitals)
    E = integrate(rho * hgh_local_potential(nuclei, elements, grid), grid)
    for i in range(orbitals.shape[-1]):
        phi = orbitals[..., i]
        E += 2.0 * inner_product(phi, hgh_nonlocal_apply(phi, nuclei, elements, grid), grid)
    return float(E + pp_nuclear_repulsion(nuclei, elements))


def bo_grad_positions(positions, charges, orbitals, elements, grid):
    """Analytic restatement of water.py:221-224 (jax.grad of bo_energy)."""
    nuclei = Nuclei(np.asarray(positions, float), np.asarray(charges, float))
    rho = _density(orbitals)
    g = hgh_local_force_density(nuclei, elements, grid, rho)
    g += hgh_nonlocal_energy_grad(nuclei, elements, grid, np.moveaxis(orbitals, -1, 0))
    g += pp_nuclear_repulsion_grad(nuclei, elements)
    return g


@dataclass
class WaterPoint:
    nuclei: Nuclei
    orbitals: np.ndarray
    energy: float
    rhf_energy: float
    nuclear_repulsion: float
    n_iters: int
    converged: bool
    orbital_energies: np.ndarray


def solve_rhf_at_geometry(nuclei, elements, grid, *, max_iters=60, tol=1e-6, mixing=0.5, order=4,
                          lanczos_iters=None, initial_orbitals=None):   # water.py:129-174
    V_local = hgh_local_potential(nuclei, elements, grid)
    n_electrons = int(total_valence_charge(elements))
    if n_electrons % 2 != 0:
        raise ValueError(f"Closed-shell RHF requires even electron count; got {n_electrons}")
    res = scf_rhf(V_local, grid, n_occ=n_electrons // 2, initial_orbitals=initial_orbitals,
                  max_iters=max_iters, tol=tol, mixing=mixing, order=order, lanczos_iters=lanczos_iters,
                  V_nl_apply=lambda p: hgh_nonlocal_apply(p, nuclei, elements, grid))
    E_nn = float(pp_nuclear_repulsion(nuclei, elements))
    return WaterPoint(nuclei, res.orbitals, float(res.energy) + E_nn, float(res.energy), E_nn,
                      res.n_iters, res.converged, res.orbital_energies)


def hellmann_feynman_force(point, elements, grid, order=4):   # water.py:227-241
    return -bo_grad_positions(point.nuclei.positions, point.nuclei.charges, point.orbitals, elements, grid)
