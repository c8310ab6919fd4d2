"""Pin the committed fixtures to the reference run with real JAX (x64), and the AO / nu
conventions to PySCF, on a machine where those are installed.

    python tests/golden/ref_parity_jax.py [path/to/GradDFT]

The fixtures in this directory are produced by make_golden.py, which runs the
reference's own modules over a torch-float64 stand-in for JAX (jaxshim.py).
Where the stand-in and JAX could differ (the gradient of jnp.clip / maximum at
an exact tie, NaN propagation through jnp.where), this script settles it:

1. With jax, jaxlib and flax importable, it imports grad_dft from the given
   checkout with x64 enabled, rebuilds each fixture's Molecule from the stored
   inputs and compares E_xc, V_xc (jax.value_and_grad, train.py:86-121) and
   the feature builders with the stored values at 1e-12 relative.
2. With pyscf importable, it builds a small molecule and compares PySCF's
   eval_gto (values, gradients, diagonal second derivatives) and int1e_grids
   with this repository's conventions (ShellBasis.from_pyscf, the oracle's
   shell evaluator and nu integrals), which the tests otherwise pin only by
   properties.

Each part prints what it checked, or that its dependency is missing; the
script exits non-zero only when a comparison fails.
"""
from __future__ import annotations

import functools
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

RTOL = 1e-12
FAILED = []


def _close(what, a, b, rtol=RTOL):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    m = ~np.isnan(b)
    ok = a.shape == b.shape and np.array_equal(np.isnan(a), np.isnan(b))
    if ok and m.any():
        scale = max(np.max(np.abs(b[m])), 1e-300)
        err = float(np.max(np.abs(a[m] - b[m])))
        ok = err <= rtol * scale
        print(f"  {what}: max abs err {err:.3e} (scale {scale:.3e}) {'ok' if ok else 'FAIL'}")
    else:
        print(f"  {what}: {'ok' if ok else 'FAIL (shape or NaN pattern)'}")
    if not ok:
        FAILED.append(what)


def jax_part(ref_root):
    try:
        import jax
        import jax.numpy as jnp
    except ImportError:
        print("jax is not importable here: the JAX x64 comparison was not run")
        return
    jax.config.update("jax_enable_x64", True)
    sys.path.insert(0, ref_root)
    try:
        import grad_dft as gd
    except ImportError as e:
        print(f"grad_dft could not be imported from {ref_root} ({e}): the JAX x64 comparison was not run")
        return
    import oracle as O

    def molecule(g):
        j = lambda x: jnp.asarray(np.asarray(x), dtype=jnp.float64)  # noqa: E731
        n = g["rdm1"].shape[1]
        grid = gd.Grid(coords=j(g["coords"]), weights=j(g["weights"]))
        return gd.Molecule(grid=grid, atom_index=jnp.zeros(1, dtype=jnp.int64), nuclear_pos=jnp.zeros((1, 3)),
                           ao=j(g["ao"]), grad_ao=j(g["grad_ao"]), grad_n_ao={1: j(g["grad_ao"]), 2: j(g["grad2_ao"])},
                           rdm1=j(g["rdm1"]), nuclear_repulsion=jnp.array(1.25), h1e=j(g["h1e"]),
                           vj=jnp.zeros((2, n, n)), mo_coeff=jnp.zeros((2, n, n)), mo_occ=jnp.zeros((2, n)),
                           mo_energy=jnp.zeros((2, n)), rep_tensor=j(g["eri"]))

    def raw_xc(functional, mol):
        def f(rdm1):
            atoms = mol.replace(rdm1=rdm1)
            dens = functional.compute_densities(atoms)
            cin = functional.compute_coefficient_inputs(atoms)
            return functional.xc_energy({"params": {}}, atoms.grid, cin, dens)

        return jax.value_and_grad(f)(mol.rdm1)

    pop, fun = gd.popular_functionals, gd.functional
    row = lambda c: (lambda self, *_: jnp.array([c]))  # noqa: E731
    functionals = {
        "LSDA": pop.LSDA, "B88": pop.B88, "VWN": pop.VWN, "LYP": pop.LYP, "PW92": pop.PW92,
        "DM21_GGA": fun.Functional(coefficients=row(O.DM21_GGA_COEFFS),
                                   energy_densities=functools.partial(fun.dm21_densities, functional_type="GGA")),
        "DM21_MGGA": fun.Functional(coefficients=row(O.DM21_MGGA_COEFFS),
                                    energy_densities=functools.partial(fun.dm21_densities, functional_type="MGGA")),
        "DENS_MGGA": fun.Functional(coefficients=row(O.DENS_MGGA_COEFFS),
                                    energy_densities=functools.partial(fun.densities, functional_type="MGGA")),
    }
    for case in ("compact", "tails"):
        g = np.load(os.path.join(HERE, f"ref_{case}.npz"))
        mol = molecule(g)
        print(f"reference with JAX x64 vs ref_{case}.npz")
        _close("rho", mol.density(), g["rho"])
        _close("tau", mol.kinetic_density(), g["tau"])
        _close("dm21_densities MGGA", fun.dm21_densities(mol, "MGGA"), g["dm21_densities_mgga"])
        _close("densities MGGA", fun.densities(mol, "MGGA"), g["densities_mgga"])
        for name, f in functionals.items():
            e, v = raw_xc(f, mol)
            _close(f"E_xc {name}", np.array(e), g[f"exc_{name}"])
            _close(f"V_xc {name}", v, g[f"vxc_{name}"])


def pyscf_part():
    try:
        from pyscf import gto
    except ImportError:
        print("pyscf is not importable here: the AO and nu convention comparison was not run")
        return
    from graddft_gb300.basis import ShellBasis
    from oracle import nu as ONU
    from oracle import shells as OS

    mol = gto.M(atom="O 0 0 0; H 0.757 0.586 0; H -0.757 0.586 0", basis="def2-tzvp", spin=0, verbose=0)
    sb = ShellBasis.from_pyscf(mol)
    spec = [(s.centre, s.l, s.exps, s.coefs, sb.rows_for(s)) for s in sb.shells]
    rng = np.random.default_rng(0)
    coords = rng.uniform(-3.0, 3.0, size=(200, 3))
    ao, g1, g2 = OS.eval_shells(spec, coords)
    ref = mol.eval_gto("GTOval_sph_deriv2", coords)  # (10, N, nao): value, x, y, z, xx, xy, xz, yy, yz, zz
    print("PySCF eval_gto vs ShellBasis.from_pyscf + the oracle's shell evaluator (H2O / def2-TZVP)")
    _close("ao", ao, ref[0], 1e-11)
    _close("grad_ao", g1, np.moveaxis(ref[1:4], 0, -1), 1e-11)
    _close("diagonal second derivatives", g2, np.stack([ref[4], ref[7], ref[9]], axis=-1), 1e-11)
    for omega in (0.0, 0.4):
        with mol.with_range_coulomb(omega):
            nu_ref = mol.intor("int1e_grids_sph", grids=coords[:20])
        nu = ONU.nu_integrals(spec, coords[:20], omega)
        _close(f"int1e_grids (omega {omega})", nu, nu_ref, 1e-10)


if __name__ == "__main__":
    jax_part(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GRADDFT_REFERENCE", ""))
    pyscf_part()
    if FAILED:
        print("FAILED:", ", ".join(FAILED))
        sys.exit(1)
