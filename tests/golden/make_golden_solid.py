"""Golden fixture of the k-point (Solid) XC path, made by running the reference's own code.

Usage (needs the reference checkout; this is not run by the tests):

    python tests/golden/make_golden_solid.py /root/reference

grad_dft/solid.py, molecule.py, functional.py, popular_functionals.py and
train.py are executed unchanged on the torch stand-ins of ``jaxshim`` (complex
tensors included; jax.grad of a real function of a complex leaf follows JAX's
convention dE/dRe - i dE/dIm).  Inputs: Bloch-phased AOs
phi_k(r) = phi(r) exp(i k.r) of a small seeded Gaussian basis with their exact
first and diagonal second derivatives, Hermitian density matrices per spin and
k-point, a Hermitian h1e and a random complex repulsion tensor.
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

import jaxshim  # noqa: E402
from oracle import shells as OS  # noqa: E402

_orig_transpose = torch.Tensor.transpose


def _transpose(self, *dims):
    if len(dims) == 1 and isinstance(dims[0], (tuple, list)):
        return self.permute(*dims[0])
    if len(dims) > 2:
        return self.permute(*dims)
    return _orig_transpose(self, *dims)


KPTS = {
    # strong phases: the unconjugated forms make some spin densities negative (NaN gradients
    # of the correlation terms, clipped to zero Fock matrices by predict)
    "solid": np.array([[0.0, 0.0, 0.0], [0.35, 0.0, 0.1], [0.0, -0.25, 0.2]]),
    # small phases over the box: positive spin densities everywhere
    "solid_small_k": np.array([[0.0, 0.0, 0.0], [0.04, -0.02, 0.0]]),
}


def solid_inputs(seed=61, n_grid=300, kpts=KPTS["solid"]):
    n_kpt = kpts.shape[0]
    g = np.random.default_rng(seed)
    shells = []
    for l in (0, 0, 1, 0):
        e = np.sort(np.exp(g.uniform(math.log(0.4), math.log(3.0), 2)))[::-1]
        shells.append((g.uniform(-1.0, 1.0, 3), l, e, OS.normalise_contraction(l, e, g.uniform(0.3, 1.0, (2, 1))),
                       None))
    coords = g.uniform(-3.0, 3.0, (n_grid, 3))
    phi, dphi, d2phi = OS.eval_shells(shells, coords)
    n = phi.shape[1]
    ph = np.exp(1j * coords @ kpts.T).T[:, :, None]  # (k, grid, 1)
    ao = phi[None] * ph
    grad_ao = (dphi[None] + 1j * kpts[:, None, None, :] * phi[None, :, :, None]) * ph[..., None]
    grad2_ao = (d2phi[None] + 2j * kpts[:, None, None, :] * dphi[None]
                - (kpts ** 2)[:, None, None, :] * phi[None, :, :, None]) * ph[..., None]
    rdm1 = np.empty((2, n_kpt, n, n), dtype=np.complex128)
    for s in range(2):
        for k in range(n_kpt):
            q, _ = np.linalg.qr(g.standard_normal((n, n)) + 1j * g.standard_normal((n, n)))
            c = q[:, :2]
            rdm1[s, k] = c @ np.diag([1.0, 0.6 + 0.2 * s]) @ c.conj().T
    h = g.standard_normal((n_kpt, n, n)) + 1j * g.standard_normal((n_kpt, n, n))
    h1e = 0.5 * (h + h.conj().transpose(0, 2, 1))
    rep = 0.02 * (g.standard_normal((n_kpt, n_kpt, n, n, n, n)) + 1j * g.standard_normal((n_kpt, n_kpt, n, n, n, n)))
    weights = g.lognormal(-2.0, 0.5, n_grid)
    kweights = np.full(n_kpt, 1.0 / n_kpt)
    return dict(coords=coords, ao=ao, grad_ao=grad_ao, grad2_ao=grad2_ao, rdm1=rdm1, h1e=h1e, rep=rep,
                weights=weights, kweights=kweights, kpts=kpts, nuclear_repulsion=np.array(1.7))


def main(root):
    torch.Tensor.transpose = _transpose
    ref = jaxshim.load_reference(root, with_solid=True)
    for case, kpts in KPTS.items():
        make_case(ref, case, solid_inputs(kpts=kpts))
    make_scf_case(ref, root)
    torch.Tensor.transpose = _orig_transpose


def make_scf_case(ref, root, cycles=4):
    """diff_simple_scf_loop (evaluate.py:256-344) on a Solid: linear mixing with the k-point predict."""
    ev = jaxshim.load_scf(root, ref)
    sol = ref.solid
    inp = solid_inputs(kpts=KPTS["solid_small_k"])
    g = np.random.default_rng(77)
    K, n = inp["rdm1"].shape[1], inp["rdm1"].shape[2]
    s1e = np.empty((K, n, n), dtype=np.complex128)
    for k in range(K):
        m = g.standard_normal((n, n)) + 1j * g.standard_normal((n, n))
        s1e[k] = np.eye(n) + 0.05 * (m @ m.conj().T) / n
    mo_occ = np.zeros((2, K, n))
    mo_occ[:, :, :2] = 1.0
    c = lambda x: torch.as_tensor(x, dtype=torch.complex128)  # noqa: E731
    f = lambda x: torch.as_tensor(x, dtype=torch.float64)  # noqa: E731
    kinfo = sol.KPointInfo(kpts_abs=f(inp["kpts"]), kpts_scaled=f(inp["kpts"]), weights=f(inp["kweights"]))
    solid = sol.Solid(grid=sol.Grid(coords=f(inp["coords"]), weights=f(inp["weights"])), kpt_info=kinfo,
                      atom_index=torch.tensor([1, 1]), lattice_vectors=f(np.eye(3) * 3.6),
                      nuclear_pos=f(np.zeros((2, 3))), ao=c(inp["ao"]), grad_ao=c(inp["grad_ao"]),
                      grad_n_ao={2: c(inp["grad2_ao"])}, rdm1=c(inp["rdm1"]),
                      nuclear_repulsion=f(inp["nuclear_repulsion"]), h1e=c(inp["h1e"]), vj=None, mo_coeff=None,
                      mo_occ=f(mo_occ), mo_energy=None, rep_tensor=c(inp["rep"]), s1e=c(s1e))
    out = dict(inp, s1e=s1e, mo_occ_init=mo_occ, cycles=np.array(cycles))
    for name in ("LSDA", "B88"):
        final = ev.diff_simple_scf_loop(getattr(ref.popular, name), cycles=cycles)({"params": {}}, solid)
        out[f"energy_{name}"] = np.asarray(final.energy.detach())
        out[f"rdm1_{name}"] = final.rdm1.detach().resolve_conj().numpy()
        out[f"fock_{name}"] = final.fock.detach().resolve_conj().numpy()
        out[f"mo_energy_{name}"] = final.mo_energy.detach().numpy()
    path = os.path.join(HERE, "ref_solid_scf.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path))


def make_case(ref, case, inp):
    sol = ref.solid
    c = lambda x: torch.as_tensor(x, dtype=torch.complex128)  # noqa: E731
    f = lambda x: torch.as_tensor(x, dtype=torch.float64)  # noqa: E731
    kinfo = sol.KPointInfo(kpts_abs=f(inp["kpts"]), kpts_scaled=f(inp["kpts"]), weights=f(inp["kweights"]))
    solid = sol.Solid(grid=sol.Grid(coords=f(inp["coords"]), weights=f(inp["weights"])), kpt_info=kinfo,
                      atom_index=torch.tensor([1, 1]), lattice_vectors=f(np.eye(3) * 3.6),
                      nuclear_pos=f(np.zeros((2, 3))), ao=c(inp["ao"]), grad_ao=c(inp["grad_ao"]),
                      grad_n_ao={2: c(inp["grad2_ao"])}, rdm1=c(inp["rdm1"]),
                      nuclear_repulsion=f(inp["nuclear_repulsion"]), h1e=c(inp["h1e"]), vj=None, mo_coeff=None,
                      mo_occ=None, mo_energy=None, rep_tensor=c(inp["rep"]))
    out = dict(inp)
    out["rho"] = solid.density().numpy()
    out["grad_rho"] = solid.grad_density().numpy()
    out["lapl"] = solid.lapl_density().numpy()
    out["tau"] = solid.kinetic_density().numpy()
    out["nonxc"] = np.asarray(solid.nonXC())
    out["vj"] = solid.get_coulomb_potential().numpy()
    for name in ("LSDA", "B88", "LYP", "PW92", "VWN"):
        E, F = ref.train.energy_predictor(getattr(ref.popular, name))({"params": {}}, solid)
        out[f"E_{name}"] = np.asarray(E.detach())
        out[f"F_{name}"] = F.detach().numpy()
    path = os.path.join(HERE, f"ref_{case}.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
