"""Host-side pieces of the SCF loop (no GPU): the safe eigensolver's reverse
rule, occupations and the density matrix, against plain torch on the CPU."""
import numpy as np
import pytest
import torch

from graddft_gb300 import scf


def test_safe_eigh_matches_torch_for_distinct_eigenvalues():
    torch.manual_seed(0)
    a = torch.randn(6, 6, dtype=torch.float64)
    a = a + a.T
    x = a.clone().requires_grad_(True)
    e, v = scf.safe_eigh(x)
    w1, w2 = torch.randn(6, dtype=torch.float64), torch.randn(6, 6, dtype=torch.float64)
    # sign-invariant functional of the eigenvectors
    ((e * w1).sum() + ((v @ v.T) * w2).sum() + ((v * v) * w2).sum()).backward()
    y = a.clone().requires_grad_(True)
    e2, v2 = torch.linalg.eigh(y)
    ((e2 * w1).sum() + ((v2 @ v2.T) * w2).sum() + ((v2 * v2) * w2).sum()).backward()
    # Away from degeneracies the broadened rule (eigenproblem.py:58-107) is the
    # ordinary symmetric-matrix eigh gradient that torch implements.
    assert torch.allclose(x.grad, y.grad, atol=1e-10), (x.grad - y.grad).abs().max()


def test_safe_eigh_degenerate_is_finite():
    a = torch.diag(torch.tensor([1.0, 1.0, 2.0], dtype=torch.float64)).requires_grad_(True)
    e, v = scf.safe_eigh(a)
    (v.sum() + e.sum()).backward()
    assert torch.isfinite(a.grad).all()


def test_general_eigh_and_occupations():
    torch.manual_seed(1)
    n = 8
    h = torch.randn(n, n, dtype=torch.float64)
    h = h + h.T
    m = torch.randn(n, n, dtype=torch.float64)
    s = torch.eye(n, dtype=torch.float64) + 0.05 * (m @ m.T) / torch.linalg.matrix_norm(m @ m.T, 2)
    e, c = scf.safe_general_eigh(h, s)
    assert torch.allclose(h @ c, s @ c @ torch.diag(e), atol=1e-10)
    assert torch.allclose(c.T @ s @ c, torch.eye(n, dtype=torch.float64), atol=1e-10)
    mo_e = torch.stack([e, e.flip(0)])
    occ = scf.get_occ(mo_e, [3, 2])
    assert occ[0, :3].sum() == 3 and occ[0, 3:].sum() == 0
    assert occ[1, -2:].sum() == 2 and occ[1, :-2].sum() == 0
    d = scf.make_rdm1(torch.stack([c, c]), occ)
    assert torch.allclose(torch.einsum("ij,ji->", d[0], s), torch.tensor(3.0, dtype=torch.float64))


def test_adam_matches_its_definition():
    """graddft_gb300.optim.adam: optax's Adam (bias-corrected moments, eps outside the square root)."""
    from graddft_gb300 import optim

    tx = optim.adam(0.05)
    w = torch.tensor([1.0, -2.0, 0.5], dtype=torch.float64)
    st = tx.init(w)
    m = v = torch.zeros(3, dtype=torch.float64)
    for k in range(1, 5):
        g = torch.tensor([0.3 * k, -0.1, 2.0 / k], dtype=torch.float64)
        u, st = tx.update(g, st, w)
        m = 0.9 * m + (1 - 0.9) * g
        v = 0.999 * v + (1 - 0.999) * g * g
        ref = -0.05 * (m / (1 - 0.9 ** k)) / (torch.sqrt(v / (1 - 0.999 ** k)) + 1e-8)
        assert torch.allclose(u, ref, rtol=1e-14, atol=0)
        w = optim.apply_updates(w, u)
    u, _ = optim.sgd(0.1).update(torch.ones(3, dtype=torch.float64), None)
    assert torch.equal(u, -0.1 * torch.ones(3, dtype=torch.float64))


def test_damping_level_shift_and_cdiis():
    """evaluate.py:1477-1545 (PySCF's damping and level shift) and the CDIIS coefficients
    (evaluate.py:1365-1385): B^-1 (1, 0, ...) by eigendecomposition equals a direct solve."""
    from graddft_gb300 import scf

    g = np.random.default_rng(3)
    n = 5
    a = g.standard_normal((n, n))
    s = torch.as_tensor(np.eye(n) + 0.1 * (a @ a.T) / n)
    d = torch.as_tensor(0.2 * np.eye(n))
    f = torch.as_tensor(g.standard_normal((n, n)))
    f = 0.5 * (f + f.T)
    f0 = (torch.eye(n, dtype=torch.float64) - s @ d) @ f @ d @ s
    assert torch.allclose(scf.damping(s, d, f, 0.25), f - (f0 + f0.T) * 0.2, rtol=1e-14, atol=1e-14)
    assert torch.allclose(scf.level_shift(s, d, f, 0.3), f + (s - s @ d @ s) * 0.3, rtol=1e-14, atol=1e-14)
    diis = scf.Diis(s, torch.eye(n, dtype=torch.float64), max_diis=3)
    errs = torch.as_tensor(g.standard_normal((3, 2, n, n)))
    x = diis.cdiis_minimize(errs)
    for sp in range(2):
        inner = torch.einsum("ikl,jkl->ij", errs[:, sp], errs[:, sp])
        B = torch.zeros((4, 4), dtype=torch.float64)
        B[1:, 1:] = inner
        B[0, 1:] = B[1:, 0] = 1.0
        rhs = torch.zeros(4, dtype=torch.float64)
        rhs[0] = 1.0
        assert torch.allclose(x[sp], torch.linalg.solve(B, rhs)[1:], rtol=1e-10, atol=1e-12)
        assert abs(float(x[sp].sum()) - 1.0) < 1e-12  # the constraint row
    with pytest.raises(NotImplementedError):
        scf.Diis(s, torch.eye(n, dtype=torch.float64), diis_method="EDIIS")


def test_canonical_eigvec_signs_and_mo_grads():
    from graddft_gb300 import scf

    g = np.random.default_rng(4)
    a = torch.as_tensor(g.standard_normal((6, 6)))
    w, v = torch.linalg.eigh(a @ a.T)
    c = scf.canonical_eigvec_signs(v)
    assert torch.allclose(c.abs(), v.abs())
    assert bool((torch.gather(c, 0, c.abs().argmax(0, keepdim=True)) > 0).all())
    assert torch.allclose(scf.canonical_eigvec_signs(-v), c)
    # mo_grads: C_vir^T F C_occ summed over spin, zeros outside the (vir, occ) block
    C = torch.as_tensor(g.standard_normal((2, 6, 6)))
    F = torch.as_tensor(g.standard_normal((2, 6, 6)))
    occ = torch.zeros((2, 6), dtype=torch.float64)
    occ[:, :2] = 1.0
    G = scf.mo_grads(C, occ, F)
    ref = sum(C[s][:, 2:].T @ F[s] @ C[s][:, :2] for s in range(2))
    assert torch.allclose(G[2:, :2], ref, rtol=1e-13, atol=1e-13)
    assert float(G[:2].abs().max()) == 0.0 and float(G[:, 2:].abs().max()) == 0.0


def test_predict_takes_cached_library_hf_terms_only():
    """predict skips the densities and inputs of train.py:165-196 only for the library's DM21 HF terms
    with dE/d ehf cached from the same predict's network pass (at the clip those terms look it up with)."""
    from graddft_gb300 import neural
    from graddft_gb300.functional import CLIP
    from graddft_gb300.train import _cached_library_hf_terms

    class Fn:
        densitygrads = neural.dm21_hfgrads_densities
        coefficient_input_grads = neural.dm21_hfgrads_cinputs

        def __init__(self, hit):
            self.hit, self.asked = hit, []

        def _hf_cached(self, params, atoms, clip):
            self.asked.append(clip)
            return ("g_dens", "g_cin") if self.hit else None

    hit = Fn(True)
    assert _cached_library_hf_terms(hit, {}, object()) and hit.asked == [CLIP]
    assert not _cached_library_hf_terms(Fn(False), {}, object())
    user = Fn(True)
    user.densitygrads = lambda *a: None  # a user-supplied term reads the arguments predict builds
    assert not _cached_library_hf_terms(user, {}, object())
    only_one = Fn(True)
    only_one.coefficient_input_grads = None
    assert _cached_library_hf_terms(only_one, {}, object())

    class NoCache:
        densitygrads = neural.dm21_hfgrads_densities
        coefficient_input_grads = None

    assert not _cached_library_hf_terms(NoCache(), {}, object())
