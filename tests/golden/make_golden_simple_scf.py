"""Golden fixture of simple_scf_loop, non_scf_predictor, scf_loop and the orbital optimisers, made by
running the reference's own code.

Usage (needs the reference checkout; this is not run by the tests):

    python tests/golden/make_golden_simple_scf.py /root/reference

grad_dft/evaluate.py (simple_scf_loop, non_scf_predictor) runs unchanged on the
torch stand-ins of ``jaxshim``.  The loop asserts at every cycle that the grid
integral of the density matches the electron count, so the synthetic system is
built to satisfy it: the seeded functions are Loewdin-orthonormalised on the grid,
the overlap is their grid overlap S = phi^T W phi (the identity to rounding), the
orbitals are S-orthonormal (core guess of a random symmetric h1e), and the
molecule has one "atom" carrying the 2 * n_occ electrons.
"""
from __future__ import annotations

import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

import jaxshim  # noqa: E402
from graddft_gb300 import synthetic  # noqa: E402
from oracle.ao_numpy import eval_ao_planes  # noqa: E402

N_GRID, N_AO, N_OCC, SEED = 600, 14, 3, 81

# jnp's transpose(perm) as predict calls it (train.py:157-162)
_orig_transpose = torch.Tensor.transpose


def _transpose(self, *dims):
    if len(dims) == 1 and isinstance(dims[0], (tuple, list)):
        return self.permute(*dims[0])
    if len(dims) > 2:  # transpose(*axes), as the Diis error matrix is built (evaluate.py:1300)
        return self.permute(*dims)
    return _orig_transpose(self, *dims)


def system():
    wl = synthetic.make_workload(N_GRID, N_AO, N_OCC, seed=SEED, box_angstrom=5.0, centre_box_angstrom=2.5)
    ao, g1, g2 = eval_ao_planes(wl.basis, wl.coords)
    w = wl.weights
    # Loewdin-orthonormalise the seeded functions on the grid (the same linear map for the
    # derivative planes), so the grid overlap is well conditioned
    e0, v0 = np.linalg.eigh(np.einsum("r,ra,rb->ab", w, ao, ao))
    X = (v0 / np.sqrt(e0)) @ v0.T
    ao, g1, g2 = ao @ X, np.einsum("rai,ab->rbi", g1, X), np.einsum("rai,ab->rbi", g2, X)
    s1e = np.einsum("r,ra,rb->ab", w, ao, ao)
    g = np.random.default_rng(SEED)
    h = g.standard_normal((N_AO, N_AO))
    h1e = 0.5 * (h + h.T) - 2.0 * np.eye(N_AO)
    eri = g.standard_normal((N_AO, N_AO, N_AO, N_AO)) * 0.002
    eri = 0.5 * (eri + eri.transpose(1, 0, 2, 3))
    eri = 0.5 * (eri + eri.transpose(0, 1, 3, 2))
    eri = 0.5 * (eri + eri.transpose(2, 3, 0, 1))
    li = np.linalg.inv(np.linalg.cholesky(s1e))
    e, v = np.linalg.eigh(li @ h1e @ li.T)
    c = li.T @ v
    mo_coeff = np.stack([c, c])
    mo_energy = np.stack([e, e])
    mo_occ = np.zeros((2, N_AO))
    mo_occ[:, :N_OCC] = 1.0
    rdm1 = np.einsum("sij,sj,skj->sik", mo_coeff, mo_occ, mo_coeff)
    return dict(ao=ao, grad_ao=g1, grad2_ao=g2, weights=w, coords=wl.coords, s1e=s1e, h1e=h1e, eri=eri,
                mo_coeff=mo_coeff, mo_energy=mo_energy, mo_occ=mo_occ, rdm1=rdm1,
                nuclear_repulsion=np.array(3.1), atom_index=np.array([2 * N_OCC]))


def orbital_system(inp, seed=SEED + 1):
    """The system in the basis phi M (M SPD, eigenvalues in [0.7, 1.4]): S = M^T S M, h and the ERIs
    transformed alike, orbitals M^-1 C (so C^T S C is unchanged) and D = M^-1 D M^-T."""
    g = np.random.default_rng(seed)
    q, _ = np.linalg.qr(g.standard_normal((N_AO, N_AO)))
    M = (q * np.linspace(0.7, 1.4, N_AO)) @ q.T
    Mi = np.linalg.inv(M)
    return dict(ao=inp["ao"] @ M, grad_ao=np.einsum("rai,ab->rbi", inp["grad_ao"], M),
                grad2_ao=np.einsum("rai,ab->rbi", inp["grad2_ao"], M), s1e=M.T @ inp["s1e"] @ M,
                h1e=M.T @ inp["h1e"] @ M, eri=np.einsum("abcd,ap,bq,cr,ds->pqrs", inp["eri"], M, M, M, M),
                mo_coeff=np.einsum("ab,sbj->saj", Mi, inp["mo_coeff"]),
                rdm1=np.einsum("ab,sbc,dc->sad", Mi, inp["rdm1"], Mi))


def _eigh_canonical(a):
    """torch.linalg.eigh with each eigenvector's largest-magnitude component positive: PCA whitening
    (evaluate.py:723-727) depends on eigenvector signs, which LAPACK builds choose differently; the
    library fixes the same convention.  Everything else the loops compute is invariant to it."""
    w, v = torch.linalg.eigh(a)
    idx = torch.argmax(v.abs(), dim=-2, keepdim=True)
    sign = torch.sign(torch.gather(v, -2, idx))
    return w, v * torch.where(sign == 0, torch.ones_like(sign), sign)


def main(root):
    torch.Tensor.transpose = _transpose
    ref = jaxshim.load_reference(root)
    ev = jaxshim.load_scf(root, ref)
    sys.modules["jax.numpy"].linalg.eigh = _eigh_canonical
    inp = system()
    t = lambda x: torch.as_tensor(np.asarray(x), dtype=torch.float64)  # noqa: E731
    mol = ref.molecule.Molecule(
        grid=ref.molecule.Grid(coords=t(inp["coords"]), weights=t(inp["weights"])),
        atom_index=torch.as_tensor(inp["atom_index"]), nuclear_pos=t(np.zeros((1, 3))), ao=t(inp["ao"]),
        grad_ao=t(inp["grad_ao"]), grad_n_ao={2: t(inp["grad2_ao"])}, rdm1=t(inp["rdm1"]),
        nuclear_repulsion=t(inp["nuclear_repulsion"]), h1e=t(inp["h1e"]), vj=None, mo_coeff=t(inp["mo_coeff"]),
        mo_occ=t(inp["mo_occ"]), mo_energy=t(inp["mo_energy"]), s1e=t(inp["s1e"]), rep_tensor=t(inp["eri"]),
        fock=t(np.zeros((2, N_AO, N_AO))), charge=0, energy=t(np.array(0.0)))
    out = dict(inp, cycles=np.array(4), mixing_factor=np.array(0.3))
    for name in ("B88", "LSDA"):
        fn = getattr(ref.popular, name)
        final = ev.simple_scf_loop(fn, mixing_factor=0.3, cycles=4)({"params": {}}, mol)
        out[f"energy_{name}"] = np.asarray(final.energy.detach())
        out[f"rdm1_{name}"] = final.rdm1.detach().numpy()
        out[f"fock_{name}"] = final.fock.detach().numpy()
        out[f"mo_energy_{name}"] = final.mo_energy.detach().numpy()
        nsp = ev.non_scf_predictor(fn)({"params": {}}, mol)
        out[f"nonscf_energy_{name}"] = np.asarray(nsp.energy.detach())
        out[f"nonscf_fock_{name}"] = nsp.fock.detach().numpy()
    # scf_loop (evaluate.py:355-592, CDIIS): all cycles, with damping + level shift, and to convergence
    runs = {"plain": dict(cycles=6, e_conv=1e-14, g_conv=1e-14),
            "shifted": dict(cycles=6, e_conv=1e-14, g_conv=1e-14, level_shift_factor=(0.1, 0.1),
                            damp_factor=(0.3, 0.3), diis_start_cycle=3),
            "converged": dict(cycles=60)}
    for key, kw in runs.items():
        final = ev.scf_loop(ref.popular.B88, **kw)({"params": {}}, mol)
        out[f"scf_{key}_energy"] = np.asarray(final.energy.detach())
        out[f"scf_{key}_rdm1"] = final.rdm1.detach().numpy()
        out[f"scf_{key}_fock"] = final.fock.detach().numpy()

    # orbital optimisers (evaluate.py:595-915) with optax.adam(1e-2), 3 steps, B88, on the same system in
    # a non-orthonormal basis (AOs times an SPD matrix M with spread eigenvalues): PCA whitening needs
    # distinct overlap eigenvalues, and the orthonormalised system's overlap is the identity
    orb = orbital_system(inp)
    mol2 = mol.replace(ao=t(orb["ao"]), grad_ao=t(orb["grad_ao"]), grad_n_ao={2: t(orb["grad2_ao"])},
                       s1e=t(orb["s1e"]), h1e=t(orb["h1e"]), rep_tensor=t(orb["eri"]), mo_coeff=t(orb["mo_coeff"]),
                       rdm1=t(orb["rdm1"]))
    out.update({f"orb/{k}": v for k, v in orb.items()})
    optax = sys.modules["optax"]
    for whitening in ("PCA", "Cholesky", "ZCA"):
        m = ev.mol_orb_optimizer(ref.popular.B88, optax.adam(1e-2), cycles=3, whitening=whitening)({"params": {}},
                                                                                                    mol2)
        out[f"orb_energy_{whitening}"] = np.asarray(m.energy.detach())
    m = ev.jitted_mol_orb_optimizer(ref.popular.B88, optax.adam(1e-2), cycles=3)({"params": {}}, mol2)
    out["orb_energy_jitted"] = np.asarray(m.energy.detach())
    torch.Tensor.transpose = _orig_transpose
    path = os.path.join(HERE, "ref_simple_scf.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
