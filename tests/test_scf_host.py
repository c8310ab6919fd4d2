"""Host-side pieces of the SCF loop (no GPU): the safe eigensolver's reverse
rule, occupations and the density matrix, against plain torch on the CPU."""
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
