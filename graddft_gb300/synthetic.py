"""Seeded synthetic inputs for the XC grid path.

The reference builds its inputs with PySCF (``interface/pyscf.py:105-201``:
``numint.eval_ao`` for the AO values, ``mf.grids`` for the quadrature grid,
``mf.make_rdm1()`` for the density matrix).  None of that is available here,
so every workload is described by a small set of seeded parameters instead:

* grid points uniform in a cube of side ``box_angstrom`` (converted to bohr
  with the reference constant ``Bohr2Angstroms = 0.52917721092``,
  ``utils/types.py:37``), weights log-normal;
* ``n_ao`` normalised Cartesian/real-solid-harmonic Gaussians
  ``phi_mu(r) = N_mu * poly_mu(r - R_mu) * exp(-alpha_mu |r - R_mu|^2)``
  with centres uniform in a smaller concentric cube, exponents log-uniform in
  ``[0.1, 50]`` bohr^-2 and angular type s/p/d with probability 1/3 each;
* ``D_sigma = C_sigma diag(occ) C_sigma^T`` with ``C_sigma`` the Q factor of a
  QR decomposition of an N(0,1) matrix and ``n_occ`` occupied orbitals.

Every array is a pure function of ``(shape, seed)``, so the device-side AO
evaluator and the CPU oracle evaluate exactly the same basis.

Random streams (one ``numpy.random.Generator(PCG64)`` each):
geometry 0, exponents/types 1, D alpha 2, D beta 3, weights 4, theta 5, ehf 6.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

BOHR2ANGSTROM = 0.52917721092  # grad_dft/utils/types.py:37

# Angular kinds and components.
S, P, D = 0, 1, 2
# p components: 0=x, 1=y, 2=z.  d components: 0=xy, 1=yz, 2=xz, 3=x^2-y^2, 4=2z^2-x^2-y^2.

STREAM_GEOMETRY, STREAM_EXPONENTS, STREAM_D_ALPHA, STREAM_D_BETA = 0, 1, 2, 3
STREAM_WEIGHTS, STREAM_THETA, STREAM_EHF = 4, 5, 6
STREAM_SCF = 7


def rng(seed: int, stream: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(np.random.SeedSequence([int(seed), int(stream)])))


@dataclass
class Basis:
    """A synthetic Gaussian basis: one primitive per AO."""

    centres: np.ndarray  # (n_ao, 3) bohr
    exponents: np.ndarray  # (n_ao,) bohr^-2
    kind: np.ndarray  # (n_ao,) int32, S/P/D
    comp: np.ndarray  # (n_ao,) int32, component within the kind
    norm: np.ndarray  # (n_ao,) analytic normalisation constant

    @property
    def n_ao(self) -> int:
        return int(self.exponents.shape[0])

    def packed(self) -> np.ndarray:
        """(n_ao, 8) float64 rows: cx, cy, cz, alpha, norm, kind, comp, 0 (device layout)."""
        out = np.zeros((self.n_ao, 8), dtype=np.float64)
        out[:, 0:3] = self.centres
        out[:, 3] = self.exponents
        out[:, 4] = self.norm
        out[:, 5] = self.kind
        out[:, 6] = self.comp
        return out


def _norm(kind: np.ndarray, comp: np.ndarray, alpha: np.ndarray) -> np.ndarray:
    """Analytic L2 normalisation of poly * exp(-alpha r^2)."""
    a = 2.0 * alpha
    i0 = (math.pi / a) ** 1.5  # int exp(-a r^2)
    n = np.empty_like(alpha)
    s = kind == S
    n[s] = 1.0 / np.sqrt(i0[s])
    p = kind == P
    n[p] = np.sqrt(2.0 * a[p] / i0[p])  # int x^2 e = i0/(2a)
    d_mixed = (kind == D) & (comp <= 2)  # xy-type: int x^2 y^2 e = i0/(4a^2)
    n[d_mixed] = 2.0 * a[d_mixed] / np.sqrt(i0[d_mixed])
    d_x2y2 = (kind == D) & (comp == 3)  # int (x^2-y^2)^2 e = i0/a^2
    n[d_x2y2] = a[d_x2y2] / np.sqrt(i0[d_x2y2])
    d_z2 = (kind == D) & (comp == 4)  # int (2z^2-x^2-y^2)^2 e = 3 i0/a^2
    n[d_z2] = a[d_z2] / np.sqrt(3.0 * i0[d_z2])
    return n


def make_basis(n_ao: int, seed: int = 0, centre_box_angstrom: float = 12.0) -> Basis:
    g = rng(seed, STREAM_GEOMETRY)
    half = 0.5 * centre_box_angstrom / BOHR2ANGSTROM
    # The grid draws from the same geometry stream after the centres.
    centres = g.uniform(-half, half, size=(n_ao, 3))
    e = rng(seed, STREAM_EXPONENTS)
    exponents = np.exp(e.uniform(math.log(0.1), math.log(50.0), size=n_ao))
    kind = e.integers(0, 3, size=n_ao).astype(np.int32)
    comp = np.zeros(n_ao, dtype=np.int32)
    comp[kind == P] = e.integers(0, 3, size=int((kind == P).sum()))
    comp[kind == D] = e.integers(0, 5, size=int((kind == D).sum()))
    return Basis(centres, exponents, kind, comp, _norm(kind, comp, exponents))


def make_grid(n_grid: int, seed: int = 0, box_angstrom: float = 20.0, n_ao_hint: int = 0):
    """Grid coordinates (n_grid, 3) in bohr and log-normal weights (n_grid,)."""
    g = rng(seed, STREAM_GEOMETRY + 100)
    half = 0.5 * box_angstrom / BOHR2ANGSTROM
    coords = g.uniform(-half, half, size=(n_grid, 3))
    w = rng(seed, STREAM_WEIGHTS).lognormal(mean=-6.0, sigma=1.0, size=n_grid)
    return coords, w


def make_rdm1(n_ao: int, n_occ: int, seed: int = 0) -> np.ndarray:
    """(2, n_ao, n_ao) projector density matrices, one per spin."""
    out = np.empty((2, n_ao, n_ao), dtype=np.float64)
    for s, stream in enumerate((STREAM_D_ALPHA, STREAM_D_BETA)):
        m = rng(seed, stream).standard_normal((n_ao, n_ao))
        q, _ = np.linalg.qr(m)
        c = q[:, :n_occ]
        out[s] = c @ c.T
    return out


def make_ehf(n_grid: int, seed: int = 0, rho: np.ndarray | None = None, n_omega: int = 2) -> np.ndarray:
    """Stop-gradient HF energy densities (omega, spin, grid).

    They stand in for ``Molecule.HF_energy_density`` (``molecule.py:504-541``),
    which needs a chi tensor made from range-separated integrals.  Values are
    scaled like the local exchange ``-1/2 rho^(4/3)`` with a seeded spread.
    """
    g = rng(seed, STREAM_EHF)
    if rho is None:
        base = np.full((2, n_grid), 1e-2)
    else:
        base = np.clip(np.asarray(rho, dtype=np.float64).T, 0.0, None)
    out = np.empty((n_omega, 2, n_grid))
    for w in range(n_omega):
        f = g.uniform(0.6, 1.0, size=(2, n_grid)) * (1.0 - 0.3 * w)
        out[w] = -0.5 * f * base ** (4.0 / 3.0)
    return out


def make_chi(ao: np.ndarray, rdm1: np.ndarray, n_omega: int = 2, seed: int = 0) -> np.ndarray:
    """A stand-in chi tensor (grid, omega, spin, orbitals) for the exact-exchange terms.

    chi^{w,s}_c(r) = sum_bd D^s_bd psi_b(r) v^w_cd(r) needs range-separated
    integrals (``interface/pyscf.py:1067-1126``); here v^w_cd(r) is replaced by a
    seeded smooth positive factor k_w (1 + 0.3 u_c(r)), so that chi = k_w (1 +
    0.3 u) (phi D) and ehf = -1/2 chi . (phi D) has the sign and rough size of
    the exchange energy density.
    """
    g = rng(seed, STREAM_EHF + 1)
    x = np.einsum("ra,sab->rsb", np.asarray(ao, dtype=np.float64), np.asarray(rdm1, dtype=np.float64))
    n_grid, _, n_ao = x.shape
    out = np.empty((n_grid, n_omega, 2, n_ao))
    for w in range(n_omega):
        k = 1.0 / (1.0 + 0.5 * w)
        u = g.uniform(-1.0, 1.0, size=(n_grid, 1, n_ao))
        out[:, w] = k * (1.0 + 0.3 * u) * x
    return out


def glorot_params(layer_widths=(256,) * 6, n_in: int = 11, n_out: int = 3, seed: int = 0) -> dict:
    """Flax-style parameter tree for the DM21 network (``functional.py:797-822``).

    Naming follows flax auto-naming in ``DM21.default_nn``: ``Dense_0`` (squash
    layer), ``Dense_1..6`` (residual), ``LayerNorm_0..5``, ``Dense_7`` (head),
    as also used by ``generate_DM21_weights`` (``functional.py:876-891``).
    Kernels are Glorot-uniform, biases small uniform, LayerNorm scale 1 and
    bias 0 plus a small seeded perturbation so every parameter is exercised.
    """
    g = rng(seed, STREAM_THETA)
    params = {}
    widths = [n_in] + list(layer_widths)

    def glorot(fan_in, fan_out):
        lim = math.sqrt(6.0 / (fan_in + fan_out))
        return g.uniform(-lim, lim, size=(fan_in, fan_out))

    params["Dense_0"] = {"kernel": glorot(n_in, widths[1]), "bias": g.uniform(-0.1, 0.1, widths[1])}
    for i in range(len(layer_widths)):
        f = layer_widths[i]
        params[f"Dense_{i + 1}"] = {"kernel": glorot(f, f), "bias": g.uniform(-0.1, 0.1, f)}
        params[f"LayerNorm_{i}"] = {
            "scale": 1.0 + g.uniform(-0.1, 0.1, f),
            "bias": g.uniform(-0.1, 0.1, f),
        }
    last = layer_widths[-1]
    params[f"Dense_{len(layer_widths) + 1}"] = {"kernel": glorot(last, n_out), "bias": g.uniform(-0.1, 0.1, n_out)}
    return {"params": params}


@dataclass
class ScfSystem:
    """One-electron data of the synthetic differentiable-SCF problem."""

    h1e: np.ndarray        # (n, n) core Hamiltonian, eigenvalues uniform in [-20, 5] Ha
    s1e: np.ndarray        # (n, n) overlap I + 0.05 M / |M|_2, M random SPD
    df_tensor: np.ndarray  # (naux, n, n) positive, symmetric in (m, n)
    rdm1: np.ndarray       # (2, n, n) core-guess density matrix
    mo_occ: np.ndarray     # (2, n) aufbau occupations of the core guess
    nuclear_repulsion: float


def make_scf_system(n_ao: int, n_occ: int, naux: int = 768, seed: int = 0) -> ScfSystem:
    """H, S, a density-fitting Coulomb tensor and the core-guess D for the SCF loop."""
    g = rng(seed, STREAM_SCF)
    q, _ = np.linalg.qr(g.standard_normal((n_ao, n_ao)))
    h = (q * g.uniform(-20.0, 5.0, n_ao)) @ q.T
    h = 0.5 * (h + h.T)
    a = g.standard_normal((n_ao, n_ao))
    m = a @ a.T + n_ao * np.eye(n_ao)
    s = np.eye(n_ao) + 0.05 * m / np.linalg.norm(m, 2)
    b = np.abs(g.standard_normal((naux, n_ao, n_ao)))
    b = 0.5 * (b + b.transpose(0, 2, 1)) / np.sqrt(naux * n_ao * n_ao)
    lc = np.linalg.cholesky(s)
    li = np.linalg.inv(lc)
    e, v = np.linalg.eigh(li @ h @ li.T)
    c = li.T @ v[:, np.argsort(e)]
    occ = np.zeros((2, n_ao))
    occ[:, :n_occ] = 1.0
    d = np.stack([(c[:, :n_occ]) @ c[:, :n_occ].T] * 2)
    # Scale B so the core-guess Coulomb matrix has entries of order 1 Ha.
    dt = d.sum(0)
    j = np.einsum("P,Pmn->mn", np.einsum("Pls,ls->P", b, dt), b)
    b *= 1.0 / np.sqrt(np.abs(j).max())
    return ScfSystem(h, s, b, d, occ, float(g.uniform(5.0, 10.0)))


@dataclass
class Workload:
    """One synthetic molecule: basis, grid, weights and density matrix."""

    basis: Basis
    coords: np.ndarray
    weights: np.ndarray
    rdm1: np.ndarray

    @property
    def n_grid(self) -> int:
        return int(self.weights.shape[0])

    @property
    def n_ao(self) -> int:
        return self.basis.n_ao


def make_workload(n_grid: int, n_ao: int, n_occ: int | None = None, seed: int = 0,
                  box_angstrom: float = 20.0, centre_box_angstrom: float = 12.0) -> Workload:
    if n_occ is None:
        n_occ = max(1, n_ao // 8)
    basis = make_basis(n_ao, seed, centre_box_angstrom)
    coords, w = make_grid(n_grid, seed, box_angstrom)
    d = make_rdm1(n_ao, n_occ, seed)
    return Workload(basis, coords, w, d)
