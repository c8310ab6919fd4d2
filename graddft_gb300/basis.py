"""Contracted Gaussian basis sets evaluated on the device.

The reference takes its AO values from PySCF: ``numint.eval_ao(mol, coords,
deriv=1)`` for phi and its gradient (``interface/pyscf.py:824, 849-852``) and
``ao_grads(mol, coords, order=2)`` for the diagonal second derivatives
(``interface/pyscf.py:677-705``).  ``ShellBasis`` describes the same functions:

    phi_{s,c,k}(r) = sum_p C[s][c][p] exp(-alpha_{s,p} |r - R_s|^2) * A_k(r - R_s)

for shell s (angular momentum l, centre R_s, primitives p, contractions c) and
angular component k, where A_k is a homogeneous polynomial of degree l:

* spherical shells (PySCF's default, ``mol.cart = False``): A_k = r^l Y_lm,
  the real solid harmonic with unit norm on the sphere and no Condon-Shortley
  phase, components ordered (x, y, z) for l = 1 and m = -l..l for l >= 2;
* cartesian shells: A_k = sqrt((2l+1)/(4 pi)) x^i y^j z^k, so that x^l, y^l
  and z^l have unit norm, ordered i = l..0 then j = l-i..0.

The AOs of a shell are ordered contraction-major, then component, and the
shells follow each other in the order given (PySCF's ``mol._bas`` order).
``normalized_contraction`` turns the coefficients of a basis-set file into
C (primitive radial normalisation, then unit norm of each contracted radial
function), the normalisation PySCF applies when it builds ``mol._env``.

Every AO carries its own row of cartesian coefficients, so any polynomial
convention (including a single component of a shell, as the seeded synthetic
basis uses) runs through the same kernel.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field
from fractions import Fraction
from typing import List, Optional, Sequence

import numpy as np

MAX_L = 6


def ncart(l: int) -> int:
    return (l + 1) * (l + 2) // 2


def cart_powers(l: int):
    """Cartesian exponents (i, j, k) of degree l in PySCF's order."""
    return [(i, j, l - i - j) for i in range(l, -1, -1) for j in range(l - i, -1, -1)]


# ------------------------------------------------------------ solid harmonics
def _dfact(n: int) -> int:
    out = 1
    while n > 1:
        out *= n
        n -= 2
    return out


def _sphere_moment(p) -> Fraction:
    """int x^a y^b z^c dOmega / (4 pi) over the unit sphere (zero unless all even)."""
    a, b, c = p
    if a % 2 or b % 2 or c % 2:
        return Fraction(0)
    return Fraction(_dfact(a - 1) * _dfact(b - 1) * _dfact(c - 1), _dfact(a + b + c + 1))


def _poly_mul(u: dict, v: dict) -> dict:
    out: dict = {}
    for pu, cu in u.items():
        for pv, cv in v.items():
            k = (pu[0] + pv[0], pu[1] + pv[1], pu[2] + pv[2])
            out[k] = out.get(k, 0) + cu * cv
    return {k: c for k, c in out.items() if c != 0}


def _solid_harmonic_poly(l: int, m: int) -> dict:
    """r^l P_l^|m|(cos theta) {cos, sin}(|m| phi) as an exact polynomial (no normalisation).

    r^l P_l^m(z/r) e^{i m phi} = (x + i y)^m * sum_k q_k z^(l-m-2k) r^(2k), with
    q_k the coefficients of d^m P_l / dt^m (Legendre's explicit sum); the real
    part gives m >= 0, the imaginary part m < 0.
    """
    am = abs(m)
    az: dict = {}
    for k in range(l // 2 + 1):
        n = l - 2 * k  # power of t in P_l
        if n < am:
            continue
        q = Fraction((-1) ** k * math.comb(l, k) * math.comb(2 * l - 2 * k, l), 2 ** l)
        q *= Fraction(math.factorial(n), math.factorial(n - am))
        kk = (n - am)  # power of z; r^(l - am - kk) = r^(2 j)
        j = (l - am - kk) // 2
        for a in range(j + 1):
            for b in range(j - a + 1):
                c = j - a - b
                coef = Fraction(math.factorial(j), math.factorial(a) * math.factorial(b) * math.factorial(c))
                p = (2 * a, 2 * b, 2 * c + kk)
                az[p] = az.get(p, 0) + q * coef
    xy: dict = {}
    for t in range(am + 1):
        if m >= 0 and t % 2 == 0:
            sign = (-1) ** (t // 2)
        elif m < 0 and t % 2 == 1:
            sign = (-1) ** ((t - 1) // 2)
        else:
            continue
        xy[(am - t, t, 0)] = Fraction(sign * math.comb(am, t))
    return _poly_mul(xy, az)


def solid_harmonic_rows(l: int) -> np.ndarray:
    """(2l+1, ncart(l)) coefficients of the unit-norm real solid harmonics on the cartesian monomials."""
    order = [1, -1, 0] if l == 1 else list(range(-l, l + 1))
    powers = cart_powers(l)
    rows = np.zeros((2 * l + 1, ncart(l)))
    for r, m in enumerate(order):
        poly = _solid_harmonic_poly(l, m)
        norm2 = sum((cu * cv * _sphere_moment((pu[0] + pv[0], pu[1] + pv[1], pu[2] + pv[2]))
                     for pu, cu in poly.items() for pv, cv in poly.items()), Fraction(0))
        scale = 1.0 / math.sqrt(4.0 * math.pi * float(norm2))
        for p, cf in poly.items():
            rows[r, powers.index(p)] = float(cf) * scale
    return rows


def cartesian_rows(l: int) -> np.ndarray:
    return math.sqrt((2 * l + 1) / (4.0 * math.pi)) * np.eye(ncart(l))


# ------------------------------------------------------------ normalisation
def _gauss_moment(n: int, a):
    """int_0^inf r^n exp(-a r^2) dr."""
    return math.gamma((n + 1) / 2.0) / (2.0 * np.asarray(a, dtype=np.float64) ** ((n + 1) / 2.0))


def normalized_contraction(l: int, exps: Sequence[float], coefs) -> np.ndarray:
    """Basis-file coefficients (nprim, nctr) -> C with unit-norm contracted radial functions.

    Each primitive r^l exp(-alpha r^2) is first normalised (int_0^inf of its
    square times r^2 is 1), then each contraction is rescaled so that
    int_0^inf R(r)^2 r^2 dr = 1 for R(r) = sum_p C_p r^l exp(-alpha_p r^2).
    """
    e = np.asarray(exps, dtype=np.float64)
    c = np.asarray(coefs, dtype=np.float64).reshape(e.shape[0], -1)
    c = c / np.sqrt(_gauss_moment(2 * l + 2, 2.0 * e))[:, None]
    s = _gauss_moment(2 * l + 2, e[:, None] + e[None, :])
    norm = np.sqrt(np.einsum("pc,pq,qc->c", c, s, c))
    return c / norm[None, :]


# ------------------------------------------------------------ the basis
@dataclass
class Shell:
    centre: np.ndarray  # (3,) bohr
    l: int
    exps: np.ndarray  # (nprim,)
    coefs: np.ndarray  # (nprim, nctr), used as given
    rows: Optional[np.ndarray] = None  # (ncomp, ncart) angular rows; default from the basis convention


@dataclass
class ShellBasis:
    shells: List[Shell]
    cart: bool = False
    _tables: dict = field(default_factory=dict, repr=False, compare=False)

    # ----------------------------------------------------------- builders
    @classmethod
    def from_pyscf(cls, mol) -> "ShellBasis":
        """Read a PySCF ``Mole`` through its documented libcint arrays.

        ``mol._bas`` rows: atom, l, nprim, nctr, kappa, exponent offset,
        coefficient offset, 0; ``mol._atm`` rows: charge, coordinate offset, ...;
        ``mol._env`` holds the coordinates (bohr), exponents and the normalised
        coefficients (contraction-major).
        """
        return cls.from_libcint(np.asarray(mol._atm), np.asarray(mol._bas), np.asarray(mol._env),
                                cart=bool(getattr(mol, "cart", False)))

    @classmethod
    def from_libcint(cls, atm, bas, env, cart: bool = False) -> "ShellBasis":
        atm = np.asarray(atm).reshape(-1, 6)
        bas = np.asarray(bas).reshape(-1, 8)
        env = np.asarray(env, dtype=np.float64)
        shells = []
        for row in bas:
            ia, l, nprim, nctr, _, pexp, pcoef = (int(v) for v in row[:7])
            if not 0 <= ia < atm.shape[0]:
                raise ValueError(f"shell refers to atom {ia} of {atm.shape[0]}")
            pc = int(atm[ia, 1])
            centre = env[pc:pc + 3].copy()
            exps = env[pexp:pexp + nprim].copy()
            coefs = env[pcoef:pcoef + nprim * nctr].reshape(nctr, nprim).T.copy()
            shells.append(Shell(centre, l, exps, coefs))
        return cls(shells, cart)

    @classmethod
    def from_synthetic(cls, basis) -> "ShellBasis":
        """The seeded single-primitive basis of ``graddft_gb300.synthetic`` (one AO per shell)."""
        rows5 = solid_harmonic_rows(2)
        # synthetic d components: xy, yz, xz, x^2-y^2, 2z^2-x^2-y^2 -> m = -2, -1, 1, 2, 0
        d_pick = [0, 1, 3, 4, 2]
        shells = []
        for a in range(basis.n_ao):
            l, comp = int(basis.kind[a]), int(basis.comp[a])
            if l == 0:
                row = solid_harmonic_rows(0)
            elif l == 1:
                row = solid_harmonic_rows(1)[comp:comp + 1]
            else:
                row = rows5[d_pick[comp]:d_pick[comp] + 1]
            # synthetic AOs are N poly exp(-alpha r^2) with their own analytic norm
            c = normalized_contraction(l, [basis.exponents[a]], [[1.0]])
            shells.append(Shell(np.asarray(basis.centres[a], dtype=np.float64), l,
                                np.asarray([basis.exponents[a]], dtype=np.float64), c, row))
        return cls(shells, cart=False)

    # ------------------------------------------------------------ shape
    def rows_for(self, sh: Shell) -> np.ndarray:
        if sh.rows is not None:
            return np.asarray(sh.rows, dtype=np.float64)
        return cartesian_rows(sh.l) if self.cart else solid_harmonic_rows(sh.l)

    @property
    def n_ao(self) -> int:
        return sum(self.rows_for(s).shape[0] * np.asarray(s.coefs).reshape(len(s.exps), -1).shape[1]
                   for s in self.shells)

    def validate(self):
        if not self.shells:
            raise ValueError("a basis needs at least one shell")
        for i, s in enumerate(self.shells):
            if not 0 <= int(s.l) <= MAX_L:
                raise ValueError(f"shell {i}: l = {s.l} outside 0..{MAX_L}")
            e = np.asarray(s.exps, dtype=np.float64)
            if e.ndim != 1 or e.size == 0 or not np.all(np.isfinite(e)) or np.any(e <= 0):
                raise ValueError(f"shell {i}: exponents must be a non-empty positive vector")
            c = np.asarray(s.coefs, dtype=np.float64)
            if c.size == 0 or c.size % e.size or not np.all(np.isfinite(c)):
                raise ValueError(f"shell {i}: coefficients must be (nprim, nctr) and finite")
            r = self.rows_for(s)
            if r.ndim != 2 or r.shape[1] != ncart(int(s.l)) or r.shape[0] == 0:
                raise ValueError(f"shell {i}: angular rows must be (ncomp, {ncart(int(s.l))})")
            if np.asarray(s.centre).shape != (3,):
                raise ValueError(f"shell {i}: centre must be 3 coordinates")

    # ------------------------------------------------------------ device
    def host_tables(self):
        """The flat tables of the C ABI's gdft_basis (numpy)."""
        self.validate()
        shell_t, centre, exps, coefs, ao_t, trans = [], [], [], [], [], []
        for i, s in enumerate(self.shells):
            e = np.asarray(s.exps, dtype=np.float64)
            c = np.asarray(s.coefs, dtype=np.float64).reshape(e.size, -1)
            rows = self.rows_for(s)
            ncomp, nctr = rows.shape[0], c.shape[1]
            shell_t.append([int(s.l), e.size, len(exps), len(coefs), len(ao_t), ncomp, nctr, len(trans)])
            centre.append(np.asarray(s.centre, dtype=np.float64))
            exps.extend(e.tolist())
            coefs.extend(c.T.reshape(-1).tolist())  # contraction-major
            trans.extend(rows.reshape(-1).tolist())
            for ic in range(nctr):
                for k in range(ncomp):
                    ao_t.append([i, ic, k, 0])
        return {
            "shell": np.asarray(shell_t, dtype=np.int32).reshape(-1, 8),
            "centre": np.asarray(centre, dtype=np.float64).reshape(-1, 3),
            "exp": np.asarray(exps, dtype=np.float64),
            "coef": np.asarray(coefs, dtype=np.float64),
            "ao": np.asarray(ao_t, dtype=np.int32).reshape(-1, 4),
            "trans": np.asarray(trans, dtype=np.float64),
        }

    def device_desc(self, device):
        """(gdft_basis, tensors) for the C ABI; the tensors own the memory the descriptor points at."""
        import torch

        from . import _lib

        key = str(device)
        if key not in self._tables:
            h = self.host_tables()
            t = {k: torch.as_tensor(v).to(device) for k, v in h.items()}
            d = _lib.GdftBasis()
            d.n_shell, d.n_ao = h["shell"].shape[0], h["ao"].shape[0]
            d.n_prim, d.n_coef, d.n_trans = h["exp"].size, h["coef"].size, h["trans"].size
            d.d_shell, d.d_centre = t["shell"].data_ptr(), t["centre"].data_ptr()
            d.d_exp, d.d_coef = t["exp"].data_ptr(), t["coef"].data_ptr()
            d.d_ao, d.d_trans = t["ao"].data_ptr(), t["trans"].data_ptr()
            self._tables[key] = (d, t)
        return self._tables[key]


def eval_ao(basis: ShellBasis, coords, deriv: int = 1, device=None):
    """numint.eval_ao (deriv 0 or 1) plus ao_grads(order=2) on the device.

    Returns ``ao`` (grid, ao), and for deriv >= 1 ``grad_ao`` (grid, ao, 3) in
    the layout the Molecule takes (``interface/pyscf.py:849-852`` moves the
    derivative axis last), and for deriv = 2 the diagonal second derivatives
    (grid, ao, 3) = ``ao_grads(...)[2]`` (``interface/pyscf.py:677-705``).
    """
    import torch

    from . import _lib, engine

    dev = engine.require_cuda(device)
    coords = engine.as_device_f64(coords, dev)
    if coords.ndim != 2 or coords.shape[1] != 3:
        raise ValueError(f"coords must be (grid, 3), got {tuple(coords.shape)}")
    if deriv not in (0, 1, 2):
        raise ValueError(f"deriv must be 0, 1 or 2, got {deriv}")
    desc, _keep = basis.device_desc(dev)
    n, nao = coords.shape[0], desc.n_ao
    ao = torch.empty((n, nao), dtype=torch.float64, device=dev)
    g1 = torch.empty((n, nao, 3), dtype=torch.float64, device=dev) if deriv >= 1 else None
    g2 = torch.empty((n, nao, 3), dtype=torch.float64, device=dev) if deriv >= 2 else None
    _lib.check(_lib.load().gdft_eval_ao(ctypes.byref(desc), engine._ptr(coords), n, deriv, engine._ptr(ao),
                                        engine._ptr(g1), engine._ptr(g2), engine._stream(dev)))
    if deriv == 0:
        return ao
    if deriv == 1:
        return ao, g1
    return ao, g1, g2


def molecule_from_basis(basis: ShellBasis, coords, weights, rdm1, precision: str = "fp64", device=None,
                        with_tables: bool = False, recompute_chunk: Optional[int] = None, **fields):
    """A Molecule whose AO tables are evaluated on the device from ``basis``.

    The stand-in for building ``ao``, ``grad_ao`` and ``grad_n_ao`` with PySCF
    in ``molecule_from_pyscf`` (``interface/pyscf.py:105-201``): the resident
    tables the XC path reads are filled straight from the shells.  With
    ``with_tables`` the reference-layout arrays are evaluated as well (the HF
    exact-exchange terms take ``ao`` from there); otherwise those fields are None.
    With ``recompute_chunk`` the tables are never held for the whole grid: each
    evaluation recomputes them chunk by chunk (``engine.ChunkedResident``).
    """
    from . import engine
    from .molecule import Grid, Molecule

    dev = engine.require_cuda(device)
    coords = engine.as_device_f64(coords, dev)
    weights = engine.as_device_f64(weights, dev)
    if recompute_chunk is not None:
        r = engine.ChunkedResident(basis, coords, weights, precision, int(recompute_chunk), dev)
    else:
        r = engine.Resident.from_shells(basis, coords, weights, precision, dev)
    ao = grad_ao = grad_n_ao = None
    if with_tables:
        ao, grad_ao, g2 = eval_ao(basis, coords, 2, dev)
        grad_n_ao = {2: g2}
    kw = dict(atom_index=None, nuclear_pos=None, nuclear_repulsion=0.0, h1e=None, vj=None, mo_coeff=None,
              mo_occ=None, mo_energy=None)
    kw.update(fields)
    return Molecule(grid=Grid(coords, weights), ao=ao, grad_ao=grad_ao, grad_n_ao=grad_n_ao,
                    rdm1=engine.as_device_f64(rdm1, dev), precision=precision, _resident=r, **kw)
