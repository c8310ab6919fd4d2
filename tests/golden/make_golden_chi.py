"""Golden fixture of generate_chi_tensor, made by running the reference's own functions.

Usage (needs the reference checkout; this is not run by the tests):

    python tests/golden/make_golden_chi.py /root/reference

``generate_chi_tensor`` (grad_dft/interface/pyscf.py) and ``_nu_chunk``
(grad_dft/external/_hf_density.py) are taken from the reference's source files
by name and executed unchanged on the torch-float64 stand-ins of ``jaxshim``.
Their only PySCF call, ``_evaluate_nu`` (int1e_grids), is replaced by the
oracle's McMurchie-Davidson integrals (oracle/nu.py): the fixture pins the
chunking, the einsum and the (grid, omega, spin, ao) layout of chi, while the
integral values are pinned by the oracle's own tests.
"""
from __future__ import annotations

import ast
import math
import os
import sys
import types

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

import jaxshim  # noqa: E402
from oracle import nu as ONU  # noqa: E402
from oracle import shells as OS  # noqa: E402


def chi_basis(seed=41):
    """Shells (centre, l, exps, coefs, rows=None) up to d, two of them contracted, one general contraction."""
    g = np.random.default_rng(seed)
    shells = []
    centres = g.uniform(-1.2, 1.2, (3, 3))
    for c in centres:
        for l, nprim, nctr in ((0, 3, 2), (1, 2, 1), (2, 1, 1)):
            e = np.sort(np.exp(g.uniform(math.log(0.3), math.log(8.0), nprim)))[::-1]
            coefs = OS.normalise_contraction(l, e, g.uniform(0.2, 1.0, (nprim, nctr)))
            shells.append((c, l, e, coefs, None))
    return shells


def _function_from(path, name, ns):
    tree = ast.parse(open(path).read(), filename=path)
    node = next(n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name == name)
    exec(compile(ast.Module(body=[node], type_ignores=[]), path, "exec"), ns)
    return ns[name]


def main(root):
    jaxshim.install()
    jax = sys.modules["jax"]
    jnp = sys.modules["jax.numpy"]
    shells = chi_basis()
    g = np.random.default_rng(42)
    n_grid = 150
    coords = g.uniform(-3.0, 3.0, (n_grid, 3))
    ao, _, _ = OS.eval_shells(shells, coords)
    n = ao.shape[1]
    rdm1 = np.stack([(lambda m: m @ m.T / n)(g.standard_normal((n, n))) for _ in range(2)])
    omegas = [0.0, 0.4]

    def evaluate_nu(mol, c, omega, hermi=True):
        return torch.as_tensor(ONU.nu_integrals(shells, np.asarray(c), omega))

    ns = {"jnp": jnp, "jax": jax, "vmap": jaxshim.vmap, "Generator": object, "Tuple": tuple, "Mole": object,
          "Array": torch.Tensor, "_evaluate_nu": evaluate_nu}
    nu_chunk = _function_from(os.path.join(root, "grad_dft", "external", "_hf_density.py"), "_nu_chunk", ns)
    ns.update({"_nu_chunk": nu_chunk, "Precision": types.SimpleNamespace(HIGHEST=None)})
    gen = _function_from(os.path.join(root, "grad_dft", "interface", "pyscf.py"), "generate_chi_tensor", ns)
    chi = gen(torch.as_tensor(rdm1), torch.as_tensor(ao), torch.as_tensor(coords), None, omegas, chunk_size=64)
    chi = np.asarray(chi)
    flat = {}
    for i, (c, l, e, cf, _) in enumerate(shells):
        flat[f"shell{i}/centre"], flat[f"shell{i}/l"] = np.asarray(c), np.array(l)
        flat[f"shell{i}/exps"], flat[f"shell{i}/coefs"] = np.asarray(e), np.asarray(cf)
    nu04 = ONU.nu_integrals(shells, coords[:16], 0.4)
    path = os.path.join(HERE, "ref_chi.npz")
    np.savez_compressed(path, coords=coords, ao=ao, rdm1=rdm1, omegas=np.asarray(omegas), chi=chi,
                        n_shell=np.array(len(shells)), nu04_first16=nu04, **flat)
    print(path, os.path.getsize(path), chi.shape)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
