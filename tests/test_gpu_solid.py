"""GPU parity of the k-point (Solid) XC path.

Solid densities (solid.py:491-632), the Coulomb potential and non-XC energy
(solid.py:272-411) and energy_predictor's (E, F) for a Solid (train.py:124-163)
against the fixture of the reference's own code (tests/golden/ref_solid.npz).
FP64 form: 1e-11 relative to the largest entry; mixed form: the molecule
path's tolerances (E 1e-6 relative, F 2e-6 of the largest entry).
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G(built_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import graddft_gb300 as G

    return G


def _close(a, b, rtol, what=""):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = np.asarray(b)
    assert a.shape == b.shape, (what, a.shape, b.shape)
    nan = np.isnan(b)
    assert np.array_equal(np.isnan(a), nan), what
    if (~nan).any():
        scale = max(np.max(np.abs(b[~nan])), 1e-300)
        err = np.max(np.abs(a[~nan] - b[~nan]))
        assert err <= rtol * scale, f"{what}: max abs err {err:.3e} vs scale {scale:.3e}"


def _solid(G, g, precision="fp64"):
    c = lambda x: torch.as_tensor(x, dtype=torch.complex128, device="cuda")  # noqa: E731
    f = lambda x: torch.as_tensor(x, dtype=torch.float64, device="cuda")  # noqa: E731
    kinfo = G.KPointInfo(kpts_abs=g["kpts"], kpts_scaled=g["kpts"], weights=g["kweights"])
    return G.Solid(grid=G.Grid(coords=f(g["coords"]), weights=f(g["weights"])), kpt_info=kinfo, atom_index=None,
                   lattice_vectors=None, nuclear_pos=None, ao=c(g["ao"]), grad_ao=c(g["grad_ao"]),
                   grad_n_ao={2: c(g["grad2_ao"])}, rdm1=c(g["rdm1"]), nuclear_repulsion=float(g["nuclear_repulsion"]),
                   h1e=c(g["h1e"]), vj=None, mo_coeff=None, mo_occ=None, mo_energy=None, rep_tensor=c(g["rep"]),
                   precision=precision)


@pytest.mark.parametrize("precision,rtol", [("fp64", 1e-11), ("tf32x3", 1e-6)])
@pytest.mark.parametrize("case", ["solid", "solid_small_k"])
def test_densities(G, golden, precision, rtol, case):
    g = golden(case)
    s = _solid(G, g, precision)
    _close(s.density(), g["rho"], rtol, "rho")
    _close(s.grad_density(), g["grad_rho"], rtol, "grad_rho")
    _close(s.lapl_density(), g["lapl"], rtol, "lapl")
    _close(s.kinetic_density(), g["tau"], rtol, "tau")


@pytest.mark.parametrize("case", ["solid", "solid_small_k"])
def test_coulomb_and_nonxc(G, golden, case):
    g = golden(case)
    s = _solid(G, g)
    _close(s.get_coulomb_potential(), g["vj"], 1e-12, "vj")
    assert abs(float(s.nonXC()) - float(g["nonxc"])) <= 1e-12 * abs(float(g["nonxc"]))


@pytest.mark.parametrize("name", ["LSDA", "B88", "LYP", "PW92", "VWN"])
@pytest.mark.parametrize("precision,rtol_e,rtol_f", [("fp64", 1e-11, 1e-11), ("tf32x3", 1e-6, 2e-6)])
@pytest.mark.parametrize("case", ["solid", "solid_small_k"])
def test_predict(G, golden, name, precision, rtol_e, rtol_f, case):
    g = golden(case)
    s = _solid(G, g, precision)
    E, F = G.energy_predictor(getattr(G, name))({"params": {}}, s)
    ref_e = float(g[f"E_{name}"])
    assert abs(float(E) - ref_e) <= rtol_e * abs(ref_e)
    _close(F, g[f"F_{name}"], rtol_f, f"F {name}")


def test_energy_and_errors(G, golden, case="solid_small_k"):
    g = golden(case)
    s = _solid(G, g)
    e = G.LSDA.energy({"params": {}}, s)
    e_xc = float(G.energy_predictor(G.LSDA)({"params": {}}, s)[0]) - float(s.nonXC())
    assert abs(float(e) - (e_xc + float(s.nonXC()))) <= 1e-12 * abs(float(e))
    with pytest.raises(NotImplementedError):
        s.select_HF_omegas([0.0])
    with pytest.raises(NotImplementedError):
        G.energy_predictor(G.B3LYP)({"params": {}}, s)
    with pytest.raises(NotImplementedError):
        G.diff_scf_loop(G.LSDA, cycles=2)({"params": {}}, s)
    with pytest.raises(ValueError):
        s.replace(rdm1=torch.zeros((2, 2, 2, 2), dtype=torch.complex128, device="cuda")).density()


@pytest.mark.parametrize("name", ["LSDA", "B88"])
@pytest.mark.parametrize("precision,rtol_e,rtol_m", [("fp64", 1e-11, 1e-9), ("tf32x3", 1e-6, 1e-5)])
def test_scf_loop(G, golden, name, precision, rtol_e, rtol_m):
    """diff_simple_scf_loop with a Solid (evaluate.py:256-344) against the reference's own loop."""
    g = golden("solid_scf")
    s = _solid(G, g, precision).replace(s1e=torch.as_tensor(g["s1e"], device="cuda"),
                                        mo_occ=torch.as_tensor(g["mo_occ_init"]))
    final = G.diff_simple_scf_loop(getattr(G, name), cycles=int(g["cycles"]))({"params": {}}, s)
    ref_e = float(g[f"energy_{name}"])
    assert abs(float(final.energy) - ref_e) <= rtol_e * abs(ref_e)
    _close(final.rdm1, g[f"rdm1_{name}"], rtol_m, "rdm1")
    _close(final.fock, g[f"fock_{name}"], rtol_m, "fock")
    _close(final.mo_energy, g[f"mo_energy_{name}"], rtol_m, "mo_energy")
