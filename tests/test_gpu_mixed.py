"""GPU parity of the mixed (TF32x3 tensor-core) form.

The density contraction rounds the AO tables and D to hi + lo TF32 pairs
(~22 bits) and accumulates in FP32 inside bounded windows, FP64 across them;
the V_xc contraction runs on block-scaled three-slice operands with exact
hi*hi chunk sums.  It is checked against the FP64 oracle on small and ragged
shapes with the tolerances below (relative to the largest entry; the largest
errors seen are about a third of them), and against the GPU FP64 form at
n_ao 512 with the absolute bounds the mixed form is specified to meet.
"""
import numpy as np
import pytest
import torch

import oracle as O
from graddft_gb300 import synthetic

pytestmark = pytest.mark.gpu

# Mixed-form tolerances, relative to the largest magnitude of the quantity.
TOL_FEAT = 2e-6
TOL_E = 5e-7
TOL_V = 2e-6
# Absolute bounds of the mixed form against the FP64 form (Ha).
ABS_DE = 1e-6
ABS_DV = 1e-7


@pytest.fixture(scope="module")
def eng(built_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from graddft_gb300 import engine

    return engine


def _rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_umma_selftest(eng):
    assert eng.selftest_umma() == 0.0


@pytest.mark.parametrize("n_ao,n_grid", [(20, 512), (64, 2048), (130, 1000), (200, 4096)])
def test_mixed_density_vs_oracle(eng, n_ao, n_grid):
    wl = synthetic.make_workload(n_grid, n_ao, max(1, n_ao // 8), seed=n_ao + 1, box_angstrom=8.0,
                                 centre_box_angstrom=5.0)
    ao, g1, g2 = O.eval_ao_planes(wl.basis, wl.coords)
    r = eng.Resident.from_tables(ao, g1, g2, wl.weights, "tf32x3")
    got = r.density(wl.rdm1)
    assert r.status() == 0
    rho, grad_rho, lapl, tau = O.features_numpy(wl.rdm1, ao, g1, g2)
    errs = {k: _rel(got[k], v) for k, v in (("rho", rho), ("grad_rho", grad_rho), ("lapl", lapl), ("tau", tau))}
    print(n_ao, n_grid, errs)
    assert all(e <= TOL_FEAT for e in errs.values()), errs


@pytest.mark.parametrize("n_ao,n_grid", [(20, 512), (64, 2048), (130, 1000), (200, 4096)])
def test_mixed_xc_vs_oracle(eng, n_ao, n_grid):
    from graddft_gb300 import _lib

    wl = synthetic.make_workload(n_grid, n_ao, max(1, n_ao // 8), seed=n_ao + 2, box_angstrom=8.0,
                                 centre_box_angstrom=5.0)
    ao, g1, g2 = O.eval_ao_planes(wl.basis, wl.coords)
    r = eng.Resident.from_tables(ao, g1, g2, wl.weights, "tf32x3")
    fn = eng.make_functional([_lib.COL_LSDA, _lib.COL_B88, _lib.COL_LYP], [1.0])
    exc, vxc = r.xc_energy_and_grads(wl.rdm1, fn)
    assert r.status() == 0
    e_ref, v_ref = O.xc_energy_and_grads("BLYP", wl.rdm1, ao, g1, g2, wl.weights)
    de = abs(float(exc) - e_ref) / abs(e_ref)
    dv = _rel(vxc, v_ref)
    print(n_ao, n_grid, "dE", de, "dV", dv, "E", e_ref, "max|V|", np.abs(v_ref).max())
    assert de <= TOL_E and dv <= TOL_V


def test_mixed_vs_fp64_gpu_large(eng):
    """n_ao 512 on 2^16 points: mixed vs the FP64 GPU form (itself pinned to the oracle)."""
    from graddft_gb300 import _lib

    wl = synthetic.make_workload(1 << 16, 512, 64, seed=0)
    fn = eng.make_functional([_lib.COL_LSDA, _lib.COL_B88, _lib.COL_LYP], [1.0])
    out = {}
    for prec in ("fp64", "tf32x3"):
        r = eng.Resident.from_basis(wl.basis.packed(), wl.coords, wl.weights, prec)
        out[prec] = r.xc_energy_and_grads(wl.rdm1, fn)
        assert r.status() == 0
        del r
    (e64, v64), (emx, vmx) = out["fp64"], out["tf32x3"]
    de = abs(float(emx) - float(e64))
    dv = float((vmx - v64).abs().max())
    print("E", float(e64), "|dE|", de, "max|V|", float(v64.abs().max()), "max|dV|", dv)
    assert de <= ABS_DE and de <= TOL_E * abs(float(e64))
    assert dv <= ABS_DV and dv <= TOL_V * float(v64.abs().max())


@pytest.mark.parametrize("case", ["compact", "tails"])
@pytest.mark.parametrize("name,fname,ftype", [("DM21_GGA", "dm21_densities", "GGA"),
                                              ("DM21_MGGA", "dm21_densities", "MGGA"),
                                              ("DENS_MGGA", "densities", "MGGA")])
def test_mixed_feature_functionals_vs_reference(eng, golden, case, name, fname, ftype):
    """The feature-power functionals (tau enters V through the kinetic term) in the mixed form against
    the reference's own E and V_xc, at the mixed form's tolerances."""
    import functools

    import graddft_gb300 as G

    g = golden(case)
    t = lambda x: torch.as_tensor(np.asarray(x), dtype=torch.float64, device="cuda")  # noqa: E731
    mol = G.Molecule(grid=G.Grid(coords=None, weights=t(g["weights"])), atom_index=None, nuclear_pos=None,
                     ao=t(g["ao"]), grad_ao=t(g["grad_ao"]), grad_n_ao={2: t(g["grad2_ao"])}, rdm1=t(g["rdm1"]),
                     nuclear_repulsion=1.25, h1e=None, vj=None, mo_coeff=None, mo_occ=None, mo_energy=None,
                     rep_tensor=None, precision="tf32x3")
    row = torch.tensor([getattr(O, name + "_COEFFS")], dtype=torch.float64)
    f = G.Functional(coefficients=lambda self, *_: row,
                     energy_densities=functools.partial(getattr(G, fname), functional_type=ftype))
    exc, vxc = f.xc_energy_and_grads({"params": {}}, mol)
    assert mol.resident().status() == 0
    e_ref = float(g[f"exc_{name}"])
    de = abs(float(exc) - e_ref) / abs(e_ref)
    dv = _rel(vxc, g[f"vxc_{name}"])
    print(case, name, "dE", de, "dV", dv)
    assert de <= TOL_E and dv <= TOL_V


def _decode_tables(r, n_grid, n_ao):
    """The mixed form's resident tables read back: point-major hi + lo, AO-major three-slice sums and
    FP32-pair sums, each as (5 or 4, n_grid, n_ao) float64 arrays (the layouts of tc_pack.cu)."""
    np_, ldk = int(r.desc.n_grid_pad), -(-n_ao // 128) * 128
    buf = r.buffer.cpu().numpy()
    a256 = lambda x: (x + 255) // 256 * 256  # noqa: E731
    plane = np_ * ldk * 4
    off_pm = a256(np_ * 8)
    off_av = a256(off_pm + 5 * 2 * plane)
    off_af = a256(off_av + 4 * 3 * plane)
    f = lambda off, n: buf[off:off + 4 * n].view(np.float32).astype(np.float64)  # noqa: E731
    pm, av, af = f(off_pm, 5 * 2 * np_ * ldk), f(off_av, 4 * 3 * np_ * ldk), f(off_af, 5 * 2 * np_ * ldk)
    p = np.arange(n_grid)[:, None]
    a = np.arange(n_ao)[None, :]

    def koff(row, k):
        return (((row >> 3) * 8 + (k >> 2)) * 128 + (row & 7) * 16 + (k & 3) * 4) // 4

    blk = 128 * 32
    nkc, npc = ldk // 32, np_ // 32
    out_pm, out_av, out_af = np.empty((5, n_grid, n_ao)), np.empty((4, n_grid, n_ao)), np.empty((5, n_grid, n_ao))
    for t in range(5):
        b = ((p // 128 * 5 + t) * nkc + a // 32) * 2
        i = b * blk + koff(p % 128, a % 32)
        out_pm[t] = pm[i] + pm[i + blk]
        b = ((a // 128 * 5 + t) * npc + p // 32) * 2
        i = b * blk + koff(a % 128, p % 32)
        out_af[t] = af[i] + af[i + blk]
        if t < 4:
            b = ((a // 128 * 4 + t) * npc + p // 32) * 3
            i = b * blk + koff(a % 128, p % 32)
            out_av[t] = (av[i] + av[i + blk]) + av[i + 2 * blk]
    return out_pm, out_av, out_af


@pytest.mark.parametrize("source", ["basis", "tables"])
def test_packed_tables_against_fp64(eng, source):
    """The mixed form's tables, built in double-float arithmetic, against FP64 values: the FP32 pairs to
    1e-10 of each AO's largest value over its 32-point chunk (about 2^-44 of the terms, which cancel in
    the gradient and Laplacian planes), the three-slice sets to 2^-31 of it, the
    point-major TF32 pairs to 2^-21 of each value.  Values below 1e-20 are measured against 1e-20: FP32
    pairs lose their low part near FP32's range (exponentials below e^-70) and flush under it."""
    n_grid, n_ao = 1000, 130
    wl = synthetic.make_workload(n_grid, n_ao, 16, seed=17, box_angstrom=8.0, centre_box_angstrom=5.0)
    ao, g1, g2 = O.eval_ao_planes(wl.basis, wl.coords)
    if source == "basis":
        r = eng.Resident.from_basis(wl.basis.packed(), wl.coords, wl.weights, "tf32x3")
    else:
        r = eng.Resident.from_tables(ao, g1, g2, wl.weights, "tf32x3")
    torch.cuda.synchronize()
    ref = np.stack([ao, g1[..., 0], g1[..., 1], g1[..., 2], g2.sum(-1)])
    pm, av, af = _decode_tables(r, n_grid, n_ao)
    # the largest magnitude of each AO over each 32-point chunk (the quantisation scale)
    pad = (-n_grid) % 32
    refp = np.pad(np.abs(ref), ((0, 0), (0, pad), (0, 0)))
    scale = np.maximum(np.repeat(refp.reshape(5, -1, 32, n_ao).max(axis=2), 32, axis=1)[:, :n_grid], 1e-20)
    err_af = np.max(np.abs(af - ref) / scale)
    err_av = np.max(np.abs(av - ref[:4]) / scale[:4])
    err_pm = np.max(np.abs(pm - ref) / np.maximum(np.abs(ref), 1e-20))
    print(source, "af", err_af, "av", err_av, "pm", err_pm)
    assert err_af <= 1e-10 and err_av <= 2.0 ** -31 and err_pm <= 2.0 ** -21, (err_af, err_av, err_pm)
