"""Benchmark of the XC grid path: E_xc forward + V_xc backward, grid points per second.

Workload (synthetic, seeded): spin 2, n_ao = 512 s/p/d Gaussians with centres
in a 12 A box, n_grid = 2^20 points in a 20 A box, log-normal weights,
D_sigma = C diag(1 x 64, 0) C^T, B88 + LYP energy densities (lsda_x + b88
correction + lyp, unit coefficients).  One step = one E_xc + V_xc evaluation
(the reference's energy_predictor.xc_energy_and_grads, train.py:86) with the
molecule resident in HBM.

    python bench.py [--gpus N --steps K --warmup W] [--form tf32x3|fp64] [--impl reference]

Prints one JSON line (rank 0).  Under torchrun the molecule has world x 2^20
grid points and each rank evaluates its own contiguous 2^20-point slice
(sharding.grid_slice; weak scaling); the per-rank partial E_xc and V_xc are
summed with one all-reduce, as the grid sum shards over points.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "E_xc fwd+bwd grid-pts/s, mixed vs FP64 form on 1 GB300 at |dE|<=1e-6 Ha"
UNIT = "grid-pts/s"
N_AO, N_GRID, N_OCC, SEED = 512, 1 << 20, 64, 0
WORKLOAD = "synthetic XC contraction: spin 2, n_ao 512 (s/p/d Gaussians), n_grid 2^20, B88+LYP, E_xc + V_xc"


def _workload(n_grid: int, n_ao: int) -> str:
    if (n_grid, n_ao) == (N_GRID, N_AO):
        return WORKLOAD
    return (f"synthetic XC contraction: spin 2, n_ao {n_ao} (s/p/d Gaussians), n_grid {n_grid}, B88+LYP, "
            "E_xc + V_xc")


def _profiled_traffic(kernel: str, n_grid: int, n_ao: int):
    """DRAM bytes per launch of a kernel, from the committed ncu summary of a smaller case.

    Traffic grows in proportion to the grid points a launch processes (each
    tile streams its own table rows), so the per-point figure of the 65,536-
    point capture is scaled to this launch.  Only the n_ao it was captured at.
    """
    path = os.path.join(ROOT, "profiles", f"{kernel}_n512_g65536.md")
    if n_ao != 512 or not os.path.exists(path):
        return None
    for ln in open(path):
        if ln.startswith("dram_bytes_per_grid_point_at_n_ao_512:"):
            return float(ln.split(":")[1]) * n_grid
    return None


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p["hbm_gbs"], p["bf16_tflops"], "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = os.path.join("/tmp", f"gdft_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(n_sample: int, threads: int, warmup: int, reps: int, n_grid: int = N_GRID, n_ao: int = N_AO):
    """The oracle (FP64 CPU restatement) on a bounded sample of the same workload: the first n_sample
    grid points, prepared once, then `warmup` untimed calls and the median of `reps` timed ones.
    Returns (points/s, median s, (workload, sample slice, E_xc, V_xc of the sample))."""
    import torch

    import oracle
    from graddft_gb300 import synthetic

    torch.set_num_threads(threads)
    wl = synthetic.make_workload(n_grid, n_ao, N_OCC, SEED)
    idx = slice(0, n_sample)
    ao, g1, g2 = oracle.eval_ao_planes(wl.basis, wl.coords[idx])
    w = wl.weights[idx]
    times = []
    for i in range(warmup + reps):
        t0 = time.perf_counter()
        e, v = oracle.xc_energy_and_grads("BLYP", wl.rdm1, ao, g1, g2, w)
        dt = time.perf_counter() - t0
        if i >= warmup:
            times.append(dt)
    med = float(np.median(times))
    return n_sample / med, med, (wl, idx, e, v)


def run_reference(args):
    """--impl reference: the reference's CPU path (oracle restatement) timed on the host cores."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    n_sample = args.cpu_sample
    value, _, (_, _, e_o, v_o) = cpu_baseline(n_sample, threads, args.warmup, args.steps, args.n_grid, args.n_ao)
    if args.dump:  # the sample's oracle E_xc and V_xc, for the GPU arm's accuracy check
        np.savez(args.dump, exc=np.array(e_o), vxc=v_o)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * n_sample / value,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": _workload(args.n_grid, args.n_ao), "n_ao": args.n_ao, "n_grid": args.n_grid,
                   "functional": "B88+LYP"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{n_sample} of the 2^20 grid points (same basis, D, weights), "
                                   "FP64 torch-CPU restatement with autograd for V_xc; median of "
                                   f"{args.steps} calls after {args.warmup} warm-ups"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


NEURAL_WORKLOAD = ("synthetic neural functional (DM21-style network, 6 x 256, 11 inputs, 3 outputs, Glorot theta): "
                   "spin 2, n_ao 256, n_grid 2^19, E_xc + V_xc + dE/dtheta")


def _neural_launches(n_layers: int) -> int:
    """Kernels one mixed neural step launches (the sequence in mlp_tc.cu plus the two contractions):
    weight packing 2 + 2n, forward 6 + 2n, backward 5 + 5n, density 2 and V_xc 3."""
    return (2 + 2 * n_layers) + (6 + 2 * n_layers) + (5 + 5 * n_layers) + 5


def run_neural(args):
    """Neural-functional forward+backward: E_xc, V_xc and dE/dtheta per step (the gradient of a
    loss (E - E_ref)^2 is 2 (E - E_ref) times these, the same kernels)."""
    import ctypes

    import torch

    from graddft_gb300 import _lib, build, engine, synthetic

    build.build()
    lib = _lib.load()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    n_grid = args.n_grid if args.n_grid != N_GRID else 1 << 19
    n_ao = args.n_ao if args.n_ao != N_AO else 256
    n_occ = max(1, n_ao // 8)
    wl = synthetic.make_workload(n_grid, n_ao, n_occ, SEED)
    rdm1 = torch.as_tensor(wl.rdm1, device=dev)
    params = synthetic.glorot_params(seed=SEED)
    net64, nettc = engine.Network(precision="fp64"), engine.Network(precision="tf32x3")
    flat = nettc.flatten(params, dev)

    def resident(prec):
        return engine.Resident.from_basis(wl.basis.packed(), wl.coords, wl.weights, prec, dev)

    r = resident("tf32x3")
    rho = r.density(rdm1, want=("rho",))["rho"].cpu().numpy()
    ehf = torch.as_tensor(synthetic.make_ehf(n_grid, SEED, rho, 2), device=dev)
    exc = torch.empty((), dtype=torch.float64, device=dev)
    vxc = torch.empty((2, n_ao, n_ao), dtype=torch.float64, device=dev)
    dp = torch.empty(nettc.n_params, dtype=torch.float64, device=dev)

    def step(res=r, net=nettc):
        res.neural_xc_energy_and_grads(rdm1, net, flat, ehf, True, True, exc, vxc, dp)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    r.status()
    lib.gdft_profile_reset()
    lib.gdft_profile_enable(1)
    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(0) as clk:
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
    lib.gdft_profile_enable(0)
    r.status()
    ms_step = e0.elapsed_time(e1) / args.steps
    stage = {}
    for name, sid in (("density", _lib.STAGE_DENSITY), ("network", _lib.STAGE_MLP), ("vxc", _lib.STAGE_VXC),
                      ("reduce", _lib.STAGE_REDUCE)):
        t, n = ctypes.c_double(), ctypes.c_int64()
        _lib.check(lib.gdft_profile_read(sid, ctypes.byref(t), ctypes.byref(n)))
        stage[name] = t.value / args.steps
    e_tc, v_tc, d_tc = exc.clone(), vxc.clone(), dp.clone()

    h_rdm1 = rdm1.cpu().pin_memory()
    h_v = torch.empty(vxc.shape, dtype=torch.float64).pin_memory()
    h_d = torch.empty(dp.shape, dtype=torch.float64).pin_memory()
    h_e = torch.empty((), dtype=torch.float64).pin_memory()
    d_rdm1 = torch.empty_like(rdm1)

    def e2e_step():
        d_rdm1.copy_(h_rdm1, non_blocking=True)
        r.neural_xc_energy_and_grads(d_rdm1, nettc, flat, ehf, True, True, exc, vxc, dp)
        h_v.copy_(vxc, non_blocking=True)
        h_d.copy_(dp, non_blocking=True)
        h_e.copy_(exc, non_blocking=True)

    for _ in range(args.warmup):
        e2e_step()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        e2e_step()
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / args.steps

    other = {}
    if not args.no_fp64:
        del r
        torch.cuda.empty_cache()
        r64 = resident("fp64")
        step(r64, net64)
        torch.cuda.synchronize()
        e0.record(stream)
        step(r64, net64)
        e1.record(stream)
        torch.cuda.synchronize()
        r64.status()
        ms64 = e0.elapsed_time(e1)
        worst = 0.0
        tree64, treetc = net64.unflatten(dp), nettc.unflatten(d_tc)
        for mod, d in tree64["params"].items():
            for leaf, g in d.items():
                worst = max(worst, float((treetc["params"][mod][leaf] - g).abs().max()) /
                            max(float(g.abs().max()), 1e-300))
        other = {"fp64_form_value": n_grid / (ms64 * 1e-3), "fp64_form_ms_per_step": ms64,
                 "mixed_over_fp64": ms64 / ms_step,
                 "accuracy_vs_fp64": {"E_xc": float(exc), "abs_dE": abs(float(e_tc) - float(exc)),
                                      "max_abs_V": float(vxc.abs().max()),
                                      "max_abs_dV": float((v_tc - vxc).abs().max()),
                                      "max_rel_dtheta_per_leaf": worst}}
    hbm, bf16, src = _peaks()
    W, L = nettc.width, nettc.n_layers
    net_flops = 2.0 * n_grid * W * (16 + L * W) + 2.0 * n_grid * L * W * W + 2.0 * n_grid * W * (16 + L * W)
    con_flops = 32.0 * n_grid * n_ao ** 2
    dom = max(("density", "network", "vxc"), key=lambda k: stage[k])
    dom_flops = {"density": con_flops / 2, "vxc": con_flops / 2, "network": net_flops}[dom]
    achieved = dom_flops / (stage[dom] * 1e-3) / 1e12
    line = {
        "metric": METRIC, "value": n_grid / (ms_step * 1e-3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "tf32x3", "data": "synthetic (seeded Gaussian basis evaluated on the device)",
        "config": {"workload": NEURAL_WORKLOAD if (n_grid, n_ao) == (1 << 19, 256) else
                   f"synthetic neural functional, n_ao {n_ao}, n_grid {n_grid}", "n_ao": n_ao, "n_grid": n_grid,
                   "network": "tf32x3 (tensor cores), FP32 activations", "contractions": "tf32x3",
                   "l2": "inputs larger than L2"},
        "roofline": {"bound": "tensor", "kernel": dom, "achieved": achieved, "peak": bf16, "unit": "TFLOP/s",
                     "frac": achieved / bf16, "peak_source": f"{src} bf16 dense (TF32 nominally half)",
                     "traffic": None, "flops_per_step": {"network": net_flops, "contractions": con_flops},
                     "stage_ms_per_step": stage},
        "e2e": {"value": n_grid / (e2e_ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": rdm1.numel() * 8,
                "d2h_bytes_per_step": vxc.numel() * 8 + dp.numel() * 8 + 8},
        "gpu_launches": _neural_launches(L) * args.steps, "clocks": clk.summary(), **other,
    }
    if not args.no_cpu:
        import oracle as O

        torch.set_num_threads(os.cpu_count() or 1)
        n_s = min(args.cpu_sample, 2048)
        ao, g1, g2 = O.eval_ao_planes(wl.basis, wl.coords[:n_s])
        t0 = time.perf_counter()
        O.xc_energy_and_grads("DM21", wl.rdm1, ao, g1, g2, wl.weights[:n_s], params=params,
                              ehf=ehf[..., :n_s].cpu().numpy(), want_param_grads=True)
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": n_s / dt, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                                "sample": f"{n_s} grid points of the same workload ({dt:.1f} s), FP64 torch-CPU "
                                          "restatement, autograd for V_xc and dE/dtheta"}
    print(json.dumps(line), flush=True)


SCF_WORKLOAD = ("differentiable SCF loop: n_ao 256, n_grid 2^19, 20 iterations, linear mixing 0.3, "
                "H eigenvalues U[-20, 5] Ha, S = I + 0.05 SPD, density-fitting J (naux 768), DM21-style network; "
                "forward loop + backward dE/dtheta through all iterations")


def run_scf(args):
    """Differentiable SCF loop (config 5 shape): loops/s, and dE/dtheta vs the FP64 form."""
    import torch

    import graddft_gb300 as G
    from graddft_gb300 import _lib, build, synthetic

    build.build()
    lib = _lib.load()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    n_grid = args.n_grid if args.n_grid != N_GRID else 1 << 19
    n_ao = args.n_ao if args.n_ao != N_AO else 256
    n_occ, cycles, mix = max(1, n_ao // 8), args.cycles, 0.3
    wl = synthetic.make_workload(n_grid, n_ao, n_occ, SEED)
    sysm = synthetic.make_scf_system(n_ao, n_occ, naux=768, seed=SEED)
    params = synthetic.glorot_params(seed=SEED)
    t = lambda x: torch.as_tensor(x, dtype=torch.float64, device=dev)  # noqa: E731

    def molecule(prec):
        r = G.engine.Resident.from_basis(wl.basis.packed(), wl.coords, wl.weights, prec, dev)
        mol = G.Molecule(grid=G.Grid(coords=None, weights=t(wl.weights)), atom_index=None, nuclear_pos=None,
                         ao=None, grad_ao=None, grad_n_ao=None, rdm1=t(sysm.rdm1), nuclear_repulsion=t(
                             sysm.nuclear_repulsion), h1e=t(sysm.h1e), vj=None, mo_coeff=None, mo_occ=t(sysm.mo_occ),
                         mo_energy=None, s1e=t(sysm.s1e), df_tensor=t(sysm.df_tensor), precision=prec, _resident=r)
        rho = r.density(t(sysm.rdm1), want=("rho",))["rho"].cpu().numpy()
        return mol.replace(ehf=t(synthetic.make_ehf(n_grid, SEED, rho, 2)))

    def run(mol, prec):
        hf = lambda atoms, *_, **__: atoms.ehf  # noqa: E731
        f = G.DM21(densitygrads=None, coefficient_input_grads=None, nograd_densities=hf,
                   nograd_coefficient_inputs=hf, precision=prec)
        leaves = {k: {kk: t(v).requires_grad_(True) for kk, v in d.items()} for k, d in params["params"].items()}
        loop = (G.diff_scf_loop(f, cycles=cycles) if args.loop == "diis"
                else G.diff_simple_scf_loop(f, cycles=cycles, mixing_factor=mix))
        out = loop({"params": leaves}, mol)
        out.energy.backward()
        return float(out.energy.detach()), leaves

    mol = molecule("tf32x3")
    for _ in range(max(1, args.warmup // 3)):
        run(mol, "tf32x3")
    torch.cuda.synchronize()
    steps = max(1, min(args.steps, 3))
    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(0) as clk:
        e0.record(stream)
        for _ in range(steps):
            e_tc, g_tc = run(mol, "tf32x3")
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    line = {
        "metric": "differentiable SCF loops/s (forward + dE/dtheta through all iterations)", "value": 1e3 / ms,
        "unit": "loops/s", "n_gpus": 1, "steps": steps, "warmup": max(1, args.warmup // 3), "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "tf32x3",
        "data": "synthetic (seeded basis, H, S, density-fitting tensor)",
        "config": {"workload": (SCF_WORKLOAD if (n_grid, n_ao, cycles, args.loop) == (1 << 19, 256, 20, "simple") else
                                f"differentiable SCF loop ({'CDIIS' if args.loop == 'diis' else 'linear mixing'}), "
                                f"n_ao {n_ao}, n_grid {n_grid}, {cycles} iterations"),
                   "n_ao": n_ao, "n_grid": n_grid, "cycles": cycles, "loop": args.loop,
                   "mixing": mix if args.loop == "simple" else None, "naux": 768,
                   "eigensolver": "FP64 generalized eigh (cuSOLVER through torch), Lorentzian-broadened reverse"},
        "grid_pts_per_s": n_grid * (cycles + 1) / (ms * 1e-3), "energy": e_tc, "clocks": clk.summary(),
    }
    if not args.no_fp64:
        del mol
        torch.cuda.empty_cache()
        mol64 = molecule("fp64")
        torch.cuda.synchronize()
        e0.record(stream)
        e_64, g_64 = run(mol64, "fp64")
        e1.record(stream)
        torch.cuda.synchronize()
        worst = max(float((g_tc[m][l].grad - g.grad).abs().max()) / max(float(g.grad.abs().max()), 1e-300)
                    for m, d in g_64.items() for l, g in d.items())
        line.update({"fp64_form_ms_per_step": e0.elapsed_time(e1), "mixed_over_fp64": e0.elapsed_time(e1) / ms,
                     "accuracy_vs_fp64": {"energy": e_64, "abs_dE": abs(e_tc - e_64),
                                          "max_rel_dtheta_per_leaf": worst}})
    print(json.dumps(line), flush=True)


BATCH_WORKLOAD = ("batched ragged training step: 64 synthetic molecules, n_ao ~ U[24, 400], n_grid = 150 n_ao "
                  "(rounded to 128), DM21-style network, loss sum_m (E_m - E_ref_m)^2, fwd+bwd (dloss/dtheta, "
                  "dloss/dD_m); one captured CUDA graph vs one molecule at a time")


def run_batch(args):
    """Config-4 shape at a tenth of its grid: batched graph replay vs one molecule at a time."""
    import ctypes

    import torch

    import graddft_gb300 as G
    from graddft_gb300 import _lib, build, engine, synthetic
    from graddft_gb300.batch import NeuralBatch

    build.build()
    lib = _lib.load()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    rng = np.random.default_rng(SEED)
    n_mol = args.n_mol
    naos = rng.integers(24, 401, size=n_mol)
    pts_per_ao = args.points_per_ao
    t = lambda x: torch.as_tensor(x, dtype=torch.float64, device=dev)  # noqa: E731
    mols = []
    for i, n_ao in enumerate(naos):
        n_grid = int(round(pts_per_ao * n_ao / 128.0)) * 128
        wl = synthetic.make_workload(n_grid, int(n_ao), max(1, int(n_ao) // 8), seed=SEED + 1 + i)
        r = engine.Resident.from_basis(wl.basis.packed(), wl.coords, wl.weights, "tf32x3", dev)
        rho = r.density(t(wl.rdm1), want=("rho",))["rho"].cpu().numpy()
        mols.append(G.Molecule(grid=G.Grid(coords=None, weights=t(wl.weights)), atom_index=None, nuclear_pos=None,
                               ao=None, grad_ao=None, grad_n_ao=None, rdm1=t(wl.rdm1), nuclear_repulsion=0.0,
                               h1e=None, vj=None, mo_coeff=None, mo_occ=None, mo_energy=None,
                               ehf=t(synthetic.make_ehf(n_grid, SEED + 100 + i, rho, 2)), precision="tf32x3",
                               _resident=r))
    hf = lambda atoms, *_, **__: atoms.ehf  # noqa: E731
    f = G.DM21(densitygrads=None, coefficient_input_grads=None, nograd_densities=hf, nograd_coefficient_inputs=hf,
               precision="tf32x3")
    params = f.init(SEED)
    b = NeuralBatch(mols, f)
    e_ref = torch.zeros(n_mol, dtype=torch.float64)
    b.step(params, eref=e_ref)
    e_ref = (b.energies.cpu() + 0.01 * torch.randn(n_mol, dtype=torch.float64,
                                                   generator=torch.Generator().manual_seed(SEED)))
    b.set_inputs(eref=e_ref)
    b.capture()
    for _ in range(args.warmup):
        b.replay()
    torch.cuda.synchronize()
    b.status()
    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(0) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            b.replay()
        e1.record(stream)
        torch.cuda.synchronize()
    ms_batch = e0.elapsed_time(e1) / args.steps
    n_pts = b.n_points

    # One molecule at a time through the same library entry, one shared workspace.
    net = f.network()
    flat = net.flatten(params, dev)
    wsb = max(ctypes.c_size_t(0).value, 0)
    for m in mols:
        nb = ctypes.c_size_t()
        _lib.check(lib.gdft_neural_workspace_bytes(ctypes.byref(m.resident().desc), ctypes.byref(net.desc),
                                                   ctypes.byref(nb)))
        wsb = max(wsb, nb.value)
    del b
    torch.cuda.empty_cache()
    ws = torch.zeros(wsb, dtype=torch.uint8, device=dev)
    exc = torch.empty(n_mol, dtype=torch.float64, device=dev)
    vx = [torch.empty((2, m.resident().n_ao, m.resident().n_ao), dtype=torch.float64, device=dev) for m in mols]
    dps = torch.empty((n_mol, net.n_params), dtype=torch.float64, device=dev)
    rd = [m._rdm1() for m in mols]

    def seq_step():
        for i, m in enumerate(mols):
            r = m.resident()
            _lib.check(lib.gdft_neural_xc_energy_and_grads(
                ctypes.byref(r.desc), engine._ptr(rd[i]), ctypes.byref(net.desc), engine._ptr(flat),
                engine._ptr(m.ehf), ctypes.c_void_p(exc.data_ptr() + 8 * i), engine._ptr(vx[i]),
                ctypes.c_void_p(dps[i].data_ptr()), engine._ptr(ws), ws.numel(), engine._stream(dev)))
        g = 2.0 * (exc - e_ref.to(dev))
        return (g[:, None] * dps).sum(0)

    for _ in range(max(1, args.warmup // 3)):
        seq_step()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(max(1, args.steps // 2)):
        seq_step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms_seq = e0.elapsed_time(e1) / max(1, args.steps // 2)
    line = {
        "metric": "batched training step molecules/s (one CUDA graph) vs one molecule at a time",
        "value": n_mol / (ms_batch * 1e-3), "unit": "molecules/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_batch, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "tf32x3", "data": "synthetic (seeded basis per molecule)",
        "config": {"workload": BATCH_WORKLOAD if (n_mol, pts_per_ao) == (64, 150) else
                   f"batched step, {n_mol} molecules, n_grid = {pts_per_ao} n_ao", "n_mol": n_mol,
                   "n_ao_range": [int(naos.min()), int(naos.max())], "grid_points_total": n_pts,
                   "grid_scale": "150 points per AO (the full 1500 per AO needs ~620 GB of resident AO tables)"},
        "grid_pts_per_s": n_pts / (ms_batch * 1e-3),
        "one_at_a_time": {"ms_per_step": ms_seq, "molecules_per_s": n_mol / (ms_seq * 1e-3),
                          "grid_pts_per_s": n_pts / (ms_seq * 1e-3)},
        "batched_over_one_at_a_time": ms_seq / ms_batch, "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


def run_stream(args):
    """Config 2 with the AO tables recomputed per grid chunk (never resident): grid-pts/s and device memory."""
    import ctypes

    import torch

    from graddft_gb300 import _lib, build, engine, synthetic

    build.build()
    lib = _lib.load()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    form = args.form or "tf32x3"
    wl = synthetic.make_workload(args.n_grid, args.n_ao, N_OCC, SEED)
    fn = engine.make_functional([_lib.COL_LSDA, _lib.COL_B88, _lib.COL_LYP], [1.0])
    rdm1 = torch.as_tensor(wl.rdm1, device=dev)
    c = engine.ChunkedResident(wl.basis.packed(), wl.coords, wl.weights, form,
                               args.chunk if args.chunk else "auto", dev)
    exc = torch.empty((), dtype=torch.float64, device=dev)
    vxc = torch.empty((2, args.n_ao, args.n_ao), dtype=torch.float64, device=dev)
    for _ in range(args.warmup):
        c.xc_energy_and_grads(rdm1, fn, None, True, exc, vxc)
    torch.cuda.synchronize()
    c.status()
    lib.gdft_profile_reset()
    lib.gdft_profile_enable(1)
    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(0) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            c.xc_energy_and_grads(rdm1, fn, None, True, exc, vxc)
        e1.record(stream)
        torch.cuda.synchronize()
    lib.gdft_profile_enable(0)
    c.status()
    ms = e0.elapsed_time(e1) / args.steps
    stage = {}
    for name, sid in (("ao", _lib.STAGE_AO), ("density", _lib.STAGE_DENSITY), ("point", _lib.STAGE_POINT),
                      ("vxc", _lib.STAGE_VXC), ("reduce", _lib.STAGE_REDUCE)):
        t, n = ctypes.c_double(), ctypes.c_int64()
        _lib.check(lib.gdft_profile_read(sid, ctypes.byref(t), ctypes.byref(n)))
        stage[name] = t.value / args.steps
    mol_bytes, ws_bytes = ctypes.c_size_t(), ctypes.c_size_t()
    _lib.check(lib.gdft_molecule_bytes(args.n_grid, args.n_ao, engine.PRECISIONS[form], ctypes.byref(mol_bytes)))
    desc = _lib.GdftMolecule()
    desc.n_grid, desc.n_ao, desc.precision = args.n_grid, args.n_ao, engine.PRECISIONS[form]
    line = {
        "metric": "E_xc fwd+bwd grid-pts/s with the AO tables recomputed per grid chunk", "value": args.n_grid / (ms * 1e-3),
        "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": form,
        "data": "synthetic (seeded Gaussian basis, evaluated per chunk on the device)",
        "config": {"workload": _workload(args.n_grid, args.n_ao) + ", AO tables recomputed per chunk",
                   "n_ao": args.n_ao, "n_grid": args.n_grid, "chunk": c.chunk, "form": form},
        "device_bytes": {"chunked_workspace": c.nbytes, "resident_tables": mol_bytes.value},
        "stage_ms_per_step": stage, "clocks": clk.summary(),
        "e_xc": float(exc),
    }
    print(json.dumps(line), flush=True)


def run_batch_full(args):
    """Config 4 at its stated grid, N = 1500 n_ao (rounded to 128): 64 molecules, n_ao ~ U[24, 400], the DM21
    network (6 x 256), loss sum_m (E_m - E_ref)^2; each molecule's AO tables recomputed per grid chunk (chunk
    size from the autotuner); E, V_xc and dE/dtheta per molecule.  Timed one molecule at a time (one workspace
    shared by all) and side by side on --streams CUDA streams (the reported value)."""
    import torch

    from graddft_gb300 import build, engine, synthetic

    build.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    rng = np.random.default_rng(SEED)
    n_mol = args.n_mol
    naos = rng.integers(24, 401, size=n_mol)
    pool = {}
    mols = []
    for i, n_ao in enumerate(naos):
        n_grid = int(round(args.points_per_ao * n_ao / 128.0)) * 128
        wl = synthetic.make_workload(n_grid, int(n_ao), max(1, int(n_ao) // 8), seed=SEED + 1 + i)
        r = engine.ChunkedResident(wl.basis.packed(), wl.coords, wl.weights, "tf32x3",
                                   args.chunk if args.chunk else "auto", dev, workspace_pool=pool)
        mols.append((r, torch.as_tensor(wl.rdm1, device=dev),
                     torch.as_tensor(synthetic.make_ehf(n_grid, SEED + 100 + i, None, 2), device=dev)))
    net = engine.Network(precision="tf32x3")
    p = synthetic.glorot_params(seed=SEED)
    flat = net.flatten({"params": {k: {kk: torch.as_tensor(v) for kk, v in d.items()}
                                   for k, d in p["params"].items()}}, dev)
    exc = torch.empty(n_mol, dtype=torch.float64, device=dev)
    vx = [torch.empty((2, r.n_ao, r.n_ao), dtype=torch.float64, device=dev) for r, _, _ in mols]
    dps = torch.empty((n_mol, net.n_params), dtype=torch.float64, device=dev)
    e_ref = torch.zeros(n_mol, dtype=torch.float64, device=dev)

    def step_one_at_a_time():
        for i, (r, d, ehf) in enumerate(mols):
            r.neural_xc_energy_and_grads(d, net, flat, ehf, want_vxc=True, want_dparams=True, exc_out=exc[i],
                                         vxc_out=vx[i], dparams_out=dps[i])
        # The caller's loss: dloss/dtheta = sum_m 2 (E_m - E_ref,m) dE_m/dtheta, dloss/dD_m = 2 (E_m - E_ref,m) V_m.
        g = 2.0 * (exc - e_ref)
        return (g[:, None] * dps).sum(0)

    step_one_at_a_time()  # tunes the chunk size per AO bucket (timed once, cached on disk)
    e_ref = exc + 0.01 * torch.randn(n_mol, dtype=torch.float64, generator=torch.Generator().manual_seed(SEED)).to(dev)
    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(step, clk=None):
        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps

    ms_one = timed(step_one_at_a_time)
    for r, _, _ in mols:
        r.status()
    # The same molecules side by side on CUDA streams, longest first to the least-loaded stream, one
    # workspace pool per stream (graddft_gb300.batch.ChunkedBatch).
    from graddft_gb300.batch import ChunkedBatch

    pool.clear()  # the one-at-a-time workspace; each stream gets its own
    torch.cuda.empty_cache()
    batch = ChunkedBatch([r for r, _, _ in mols], n_streams=args.streams)
    rdm1s, ehfs = [d for _, d, _ in mols], [e for _, _, e in mols]

    def step():
        batch.neural_xc_energy_and_grads(rdm1s, net, flat, ehfs, exc, vx, dps)
        g = 2.0 * (exc - e_ref)
        return (g[:, None] * dps).sum(0)

    with Clocks(0) as clk:
        ms = timed(step)
    batch.status()
    pool = {i: w for i, p in enumerate(batch.pools) for w in p.values()}
    n_pts = sum(r.n_grid for r, _, _ in mols)
    line = {
        "metric": "batched training step molecules/s at the full config-4 grid (AO tables recomputed per chunk)",
        "value": n_mol / (ms * 1e-3), "unit": "molecules/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "tf32x3", "data": "synthetic (seeded basis per molecule)",
        "config": {"workload": f"batched step, {n_mol} molecules, n_ao ~ U[24, 400], n_grid = "
                               f"{args.points_per_ao} n_ao, DM21 network 6 x 256", "n_mol": n_mol,
                   "n_ao_range": [int(naos.min()), int(naos.max())], "grid_points_total": n_pts,
                   "chunks": sorted({int(r.chunk) for r, _, _ in mols}), "streams": len(batch.streams)},
        "grid_pts_per_s": n_pts / (ms * 1e-3), "device_bytes_workspace": sum(w.numel() for w in pool.values()),
        "one_at_a_time": {"ms_per_step": ms_one, "molecules_per_s": n_mol / (ms_one * 1e-3),
                          "grid_pts_per_s": n_pts / (ms_one * 1e-3)},
        "streams_over_one_at_a_time": ms_one / ms,
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


def run_hf(args):
    """DM21 energy_predictor with its exact-exchange terms from a chi tensor: grid-pts/s of (E, Fock)."""
    import time

    import torch

    import graddft_gb300 as G
    import oracle as O
    from graddft_gb300 import build, synthetic

    build.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    n_grid = args.n_grid if args.n_grid != N_GRID else 1 << 17
    n_ao = args.n_ao if args.n_ao != N_AO else 128
    wl = synthetic.make_workload(n_grid, n_ao, max(1, n_ao // 8), SEED)
    t = lambda x: torch.as_tensor(np.asarray(x), dtype=torch.float64, device=dev)  # noqa: E731
    form = args.form or "fp64"
    r = G.engine.Resident.from_basis(wl.basis.packed(), wl.coords, wl.weights, "fp64", dev)
    ao = r.ao_planes()[0, :n_grid, :n_ao].contiguous()  # phi as evaluated on the device
    if form == "tf32x3":  # density, V_xc, exchange contractions and network in the mixed form
        r = G.engine.Resident.from_basis(wl.basis.packed(), wl.coords, wl.weights, "tf32x3", dev)
    chi = synthetic.make_chi(ao.cpu().numpy(), wl.rdm1, n_omega=2, seed=SEED)
    rng = np.random.default_rng(SEED)
    h = rng.standard_normal((n_ao, n_ao))
    eri = rng.standard_normal((n_ao, n_ao, n_ao, n_ao)) * (0.01 / n_ao)
    mol = G.Molecule(grid=G.Grid(coords=None, weights=t(wl.weights)), atom_index=None, nuclear_pos=None, ao=ao,
                     grad_ao=None, grad_n_ao=None, rdm1=t(wl.rdm1), nuclear_repulsion=1.0, h1e=t(0.5 * (h + h.T)),
                     vj=None, mo_coeff=None, mo_occ=None, mo_energy=None, rep_tensor=t(eri), omegas=[0.0, 0.4],
                     chi=t(chi), precision=form, _resident=r)
    params = synthetic.glorot_params(seed=SEED)
    predict = G.energy_predictor(G.DM21(precision=form))
    for _ in range(max(1, args.warmup)):
        predict(params, mol)
    torch.cuda.synchronize()
    steps = max(1, min(args.steps, 5))
    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(0) as clk:
        e0.record(stream)
        for _ in range(steps):
            E, F = predict(params, mol)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    line = {
        "metric": "DM21 predict with exact-exchange terms from chi, grid-pts/s (E, Fock)", "value": n_grid / (ms * 1e-3),
        "unit": "grid-pts/s", "n_gpus": 1, "steps": steps, "warmup": max(1, args.warmup), "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64" if form == "fp64" else form,
        "data": "synthetic (seeded basis, rdm1, stand-in chi tensor, random symmetric h1e and eri)",
        "config": {"workload": f"DM21 energy_predictor with chi: n_ao {n_ao}, n_grid {n_grid}, omegas (0, 0.4)",
                   "n_ao": n_ao, "n_grid": n_grid,
                   "network": "DM21 6 x 256, " + ("FP64 form" if form == "fp64" else "TF32x3 tensor-core form"),
                   "exchange": ("FP64 GEMMs" if form == "fp64" else
                                "block-scaled three-slice tcgen05 GEMMs (ao.[D0|D1], ao^T [B0|B1])"),
                   "form": form,
                   "l2": "inputs larger than L2 (chi %.2f GiB)" % (chi.nbytes / 2**30)},
        "clocks": clk.summary(),
    }
    if not args.no_cpu:
        n_s = min(args.cpu_sample, 2048)
        sl = slice(0, n_s)
        g1 = O.eval_ao_planes(wl.basis, wl.coords[sl])
        torch.set_num_threads(os.cpu_count() or 1)
        t0 = time.perf_counter()
        O.xc_energy_and_grads("DM21", wl.rdm1, g1[0], g1[1], g1[2], wl.weights[sl], params=params,
                              ehf=O.hf_energy_density(wl.rdm1, g1[0], chi[sl]))
        O.dm21_hf_fock_terms(wl.rdm1, g1[0], g1[1], g1[2], wl.weights[sl], params, chi[sl])
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": n_s / dt, "unit": "grid-pts/s", "cores": os.cpu_count(), "kind": "port",
                                "sample": f"{n_s} grid points of the same workload ({dt:.1f} s), FP64 torch-CPU "
                                          "restatement of E_xc, V_xc and both HF Fock terms"}
    print(json.dumps(line))


def contracted_basis(n_atoms: int, seed: int = SEED):
    """A seeded contracted spherical basis: per atom s(6 prim) + 3 s, p(3 prim) + 2 p, 2 d, 1 f (30 AOs),
    centres uniform in a 12 A box, exponents log-uniform (tight contracted primitives up to 5000 bohr^-2)."""
    import math

    from graddft_gb300 import basis as B
    from graddft_gb300 import synthetic

    g = synthetic.rng(seed, 20)
    half = 0.5 * 12.0 / synthetic.BOHR2ANGSTROM
    pattern = [(0, 6), (0, 1), (0, 1), (0, 1), (1, 3), (1, 1), (1, 1), (2, 1), (2, 1), (3, 1)]
    shells = []
    for _ in range(n_atoms):
        centre = g.uniform(-half, half, 3)
        for l, nprim in pattern:
            top = 5000.0 if nprim > 1 else 20.0
            e = np.sort(np.exp(g.uniform(math.log(0.1), math.log(top), nprim)))[::-1]
            shells.append(B.Shell(centre, l, e, B.normalized_contraction(l, e, g.uniform(0.1, 1.0, (nprim, 1)))))
    return B.ShellBasis(shells)


def run_ao(args):
    """AO evaluation from contracted shells into the resident tables (numint.eval_ao + ao_grads on the device)."""
    import ctypes

    import torch

    from oracle import shells as OS
    from graddft_gb300 import _lib, build, engine, synthetic

    build.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    n_grid = args.n_grid
    n_atoms = max(1, args.n_ao // 30)
    basis = contracted_basis(n_atoms)
    n_ao = basis.n_ao
    coords, w = synthetic.make_grid(n_grid, SEED)
    form = args.form or "fp64"
    r = engine.Resident(n_grid, n_ao, form, dev)
    desc, _keep = basis.device_desc(dev)
    c_d = torch.as_tensor(coords, device=dev)
    w_d = torch.as_tensor(w, device=dev)
    lib = _lib.load()
    stream = torch.cuda.current_stream(dev)
    sp = engine._stream(dev)

    def step():
        _lib.check(lib.gdft_molecule_eval_shells(ctypes.byref(r.desc), ctypes.byref(desc), engine._ptr(c_d),
                                                 engine._ptr(w_d), sp))

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    steps = max(1, args.steps)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(0) as clk:
        e0.record(stream)
        for _ in range(steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    np_, ld = int(r.desc.n_grid_pad), int(r.desc.ld)
    ldk = (n_ao + 127) // 128 * 128
    # algorithmic bytes written per launch: the resident tables of the form
    out_bytes = 5 * np_ * ld * 8 if form == "fp64" else (5 * 2 + 4 * 3 + 5) * np_ * ldk * 4
    hbm, _, src = _peaks()
    n_exp = sum(len(s.exps) * (2 * s.l + 1) for s in basis.shells)
    line = {
        "metric": "AO tables from contracted shells (phi, grad phi, lap phi), grid-pts/s", "value": n_grid / (ms * 1e-3),
        "unit": "grid-pts/s", "n_gpus": 1, "steps": steps, "warmup": max(3, args.warmup), "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded contracted spherical basis, uniform grid)",
        "config": {"workload": f"gdft_molecule_eval_shells: {n_atoms} atoms x (4s 3p 2d 1f) = {n_ao} AOs, "
                               f"n_grid {n_grid}, {form} tables", "n_ao": n_ao, "n_grid": n_grid, "form": form,
                   "exp_per_point": n_exp, "l2": "output tables larger than L2"},
        "roofline": {"bound": "hbm", "achieved": out_bytes / (ms * 1e-3) / 1e9, "peak": hbm, "unit": "GB/s",
                     "frac": out_bytes / (ms * 1e-3) / 1e9 / hbm, "traffic": None,
                     "note": f"bytes written by the table pass over its duration, of {src} copy bandwidth; "
                             f"{n_exp} FP64 exponentials per point"},
        "clocks": clk.summary(),
    }
    if not args.no_cpu:
        n_s = min(args.cpu_sample, 1024)
        spec = [(s.centre, s.l, s.exps, s.coefs, None) for s in basis.shells]
        t0 = time.perf_counter()
        OS.eval_shells(spec, coords[:n_s])
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": n_s / dt, "unit": "grid-pts/s", "cores": 1, "kind": "port",
                                "sample": f"{n_s} grid points ({dt:.1f} s), numpy restatement (oracle/shells.py) "
                                          "of phi, grad phi and the diagonal second derivatives"}
    print(json.dumps(line))


def run_chi(args):
    """chi for DM21's two omegas (generate_chi_tensor) from an l <= 2 contracted basis: grid-pts/s."""
    import torch

    from oracle import nu as ONU
    from oracle import shells as OS
    from graddft_gb300 import build, chi, synthetic
    from graddft_gb300 import basis as B

    build.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    n_grid = args.n_grid if args.n_grid != N_GRID else 1 << 16
    n_atoms = max(1, (args.n_ao if args.n_ao != N_AO else 128) // 23)
    full = contracted_basis(n_atoms)
    basis = B.ShellBasis([s for s in full.shells if s.l <= 2])  # per atom 4 s, 3 p, 2 d = 23 AOs
    n_ao = basis.n_ao
    coords, w = synthetic.make_grid(n_grid, SEED)
    g = np.random.default_rng(SEED)
    m = g.standard_normal((2, n_ao, n_ao))
    rdm1 = np.einsum("sab,scb->sac", m, m) / n_ao
    c_d = torch.as_tensor(coords, device=dev)
    ao = B.eval_ao(basis, c_d, deriv=0)
    rdm1_d = torch.as_tensor(rdm1, device=dev)
    omegas = [0.0, 0.4]
    chunk = 4096

    def step():
        return chi.generate_chi_tensor(rdm1_d, ao, c_d, basis, omegas, chunk_size=chunk)

    for _ in range(max(1, args.warmup)):
        step()
    torch.cuda.synchronize()
    steps = max(1, min(args.steps, 3))
    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(0) as clk:
        e0.record(stream)
        for _ in range(steps):
            out = step()
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    n_pp = sum(len(a.exps) * len(b.exps) for i, a in enumerate(basis.shells) for b in basis.shells[:i + 1])
    line = {
        "metric": "chi tensor (generate_chi_tensor, omegas 0 and 0.4), grid-pts/s", "value": n_grid / (ms * 1e-3),
        "unit": "grid-pts/s", "n_gpus": 1, "steps": steps, "warmup": max(1, args.warmup), "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded contracted basis up to d, random positive semi-definite rdm1, uniform grid)",
        "config": {"workload": f"generate_chi_tensor: {n_atoms} atoms x (4s 3p 2d) = {n_ao} AOs, n_grid {n_grid}, "
                               f"omegas (0, 0.4), chunk {chunk}", "n_ao": n_ao, "n_grid": n_grid,
                   "primitive_pairs": n_pp, "chi_gib": out.numel() * 8 / 2**30},
        "clocks": clk.summary(),
    }
    if not args.no_cpu:
        n_s = 8
        spec = [(s.centre, s.l, s.exps, s.coefs, None) for s in basis.shells]
        t0 = time.perf_counter()
        a_s, _, _ = OS.eval_shells(spec, coords[:n_s])
        ONU.generate_chi(rdm1, a_s, [ONU.nu_integrals(spec, coords[:n_s], wv) for wv in omegas])
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": n_s / dt, "unit": "grid-pts/s", "cores": 1, "kind": "port",
                                "sample": f"{n_s} grid points ({dt:.1f} s), numpy McMurchie-Davidson restatement "
                                          "(oracle/nu.py) and the reference's chi einsum"}
    print(json.dumps(line))


def run_solid(args):
    """k-point (Solid) E_xc + complex V_xc for B88+LYP: grid-pts/s over all k-points."""
    import torch

    import oracle.solid as OSd
    from graddft_gb300 import basis as B
    from graddft_gb300 import build, engine, synthetic, _lib
    from graddft_gb300.solid import KPointResident

    build.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    n_grid = args.n_grid if args.n_grid != N_GRID else 1 << 17
    n_ao = args.n_ao if args.n_ao != N_AO else 64
    n_kpt = 4
    form = args.form or "tf32x3"
    wl = synthetic.make_workload(n_grid, n_ao, max(1, n_ao // 8), SEED)
    sb = B.ShellBasis.from_synthetic(wl.basis)
    c_d = torch.as_tensor(wl.coords, device=dev)
    phi, dphi, d2phi = B.eval_ao(sb, c_d, deriv=2)
    kpts = torch.tensor([[0.0, 0.0, 0.0], [0.02, 0.0, 0.0], [0.0, 0.02, 0.0], [0.0, 0.0, 0.02]],
                        dtype=torch.float64, device=dev)[:n_kpt]
    ph = torch.exp(1j * (c_d @ kpts.T)).T[:, :, None]  # Bloch phases (k, grid, 1)
    kk = kpts[:, None, None, :]
    ao = phi[None] * ph
    grad_ao = (dphi[None] + 1j * kk * phi[None, :, :, None]) * ph[..., None]
    grad2_ao = (d2phi[None] + 2j * kk * dphi[None] - kk * kk * phi[None, :, :, None]) * ph[..., None]
    del phi, dphi, d2phi
    g = np.random.default_rng(SEED)
    rdm1 = np.empty((2, n_kpt, n_ao, n_ao), dtype=np.complex128)
    for s in range(2):
        for k in range(n_kpt):
            q, _ = np.linalg.qr(g.standard_normal((n_ao, n_ao)) + 1j * g.standard_normal((n_ao, n_ao)))
            c = q[:, :max(1, n_ao // 8)]
            rdm1[s, k] = c @ c.conj().T
    kw = np.full(n_kpt, 1.0 / n_kpt)
    res = KPointResident(ao, grad_ao, grad2_ao, torch.as_tensor(wl.weights, device=dev), kw, form, dev)
    d_rdm1 = torch.as_tensor(rdm1, device=dev)
    fn = engine.make_functional([_lib.COL_LSDA, _lib.COL_B88, _lib.COL_LYP], [1.0])

    def step():
        return res.xc_energy_and_grads(d_rdm1, fn)

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    steps = max(1, args.steps)
    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(0) as clk:
        e0.record(stream)
        for _ in range(steps):
            exc, vxc = step()
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    line = {
        "metric": "Solid E_xc + complex V_xc (all k-points), grid-pts/s", "value": n_grid / (ms * 1e-3),
        "unit": "grid-pts/s", "n_gpus": 1, "steps": steps, "warmup": max(3, args.warmup), "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64" if form == "fp64" else "tf32x3",
        "data": "synthetic (seeded Gaussians with Bloch phases, Hermitian density matrices per k-point)",
        "config": {"workload": f"k-point XC: {n_kpt} k-points x {n_ao} crystal AOs, n_grid {n_grid}, B88+LYP, "
                               f"{form} form", "n_kpt": n_kpt, "n_ao": n_ao, "n_grid": n_grid, "form": form},
        "clocks": clk.summary(),
    }
    if not args.no_cpu:
        n_s = min(args.cpu_sample, 4096)
        sl = slice(0, n_s)
        t0 = time.perf_counter()
        e_ref, _ = OSd.solid_xc_energy_and_grads("BLYP", rdm1, ao[:, sl].cpu().numpy(), grad_ao[:, sl].cpu().numpy(),
                                                 grad2_ao[:, sl].cpu().numpy(), wl.weights[sl], kw)
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": n_s / dt, "unit": "grid-pts/s", "cores": os.cpu_count(), "kind": "port",
                                "sample": f"{n_s} grid points ({dt:.1f} s), torch-CPU restatement of the k-point "
                                          "densities, BLYP and the complex jax.grad (oracle/solid.py)"}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="mine", choices=["mine", "reference"])
    ap.add_argument("--form", default=None, choices=["tf32x3", "fp64"])
    ap.add_argument("--n-grid", type=int, default=N_GRID)
    ap.add_argument("--n-ao", type=int, default=N_AO)
    ap.add_argument("--fp64-grid", type=int, default=1 << 16,
                    help="grid points of the FP64-form measurement (its rate is per point)")
    ap.add_argument("--cpu-sample", type=int, default=4096)
    ap.add_argument("--seeds", type=int, default=3, help="seeded workloads of the mixed-vs-FP64 accuracy check")
    ap.add_argument("--dump", default=None, help="--impl reference: write the sample's oracle E_xc, V_xc here")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64-form run (rate and accuracy)")
    ap.add_argument("--workload", default="xc",
                    choices=["xc", "neural", "scf", "batch", "batch_full", "stream", "hf", "ao", "chi", "solid"],
                    help="xc: B88+LYP contraction benchmark (headline); neural: DM21-style network fwd+bwd; "
                         "scf: differentiable SCF loop; batch: many molecules per step; hf: DM21 predict with "
                         "its exact-exchange terms from a chi tensor; ao: AO tables from contracted shells; chi: the chi tensor from range-separated integrals; solid: k-point XC for a Solid")
    ap.add_argument("--n-mol", type=int, default=64, help="molecules (--workload batch)")
    ap.add_argument("--chunk", type=int, default=None,
                    help="grid points per chunk of --workload stream / batch_full (default: the autotuner's choice)")
    ap.add_argument("--points-per-ao", type=int, default=150, help="grid points per AO (--workload batch)")
    ap.add_argument("--streams", type=int, default=3, help="CUDA streams of --workload batch_full")
    ap.add_argument("--cycles", type=int, default=20, help="SCF iterations (--workload scf)")
    ap.add_argument("--loop", default="simple", choices=["simple", "diis"],
                    help="--workload scf: linear density mixing (diff_simple_scf_loop) or CDIIS (diff_scf_loop)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "neural":
        return run_neural(args)
    if args.workload == "scf":
        return run_scf(args)
    if args.workload == "batch":
        return run_batch(args)
    if args.workload == "batch_full":
        if args.points_per_ao == 150:
            args.points_per_ao = 1500
        return run_batch_full(args)
    if args.workload == "stream":
        return run_stream(args)
    if args.workload == "hf":
        return run_hf(args)
    if args.workload == "ao":
        return run_ao(args)
    if args.workload == "chi":
        return run_chi(args)
    if args.workload == "solid":
        return run_solid(args)

    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from graddft_gb300 import _lib, build, engine, synthetic

    build.build()
    lib = _lib.load()
    form = args.form or "tf32x3"
    dev = torch.device("cuda", local)
    fn = engine.make_functional([_lib.COL_LSDA, _lib.COL_B88, _lib.COL_LYP], [1.0])

    # One molecule of world * n_grid points; each rank owns its contiguous n_grid-point slice
    # (sharding.grid_slice: weak scaling, per-rank work fixed as the world grows).
    from graddft_gb300 import sharding

    def workload(seed):
        wl_ = synthetic.make_workload(world * args.n_grid, args.n_ao, N_OCC, seed)
        a, b = sharding.grid_slice(world * args.n_grid, rank, world)
        return wl_, slice(a, b)

    wl, mine = workload(SEED)
    rdm1 = torch.as_tensor(wl.rdm1, device=dev)

    def resident(precision, wl_=None, sl=None):
        wl_, sl = (wl, mine) if wl_ is None else (wl_, sl)
        return engine.Resident.from_basis(wl_.basis.packed(), wl_.coords[sl], wl_.weights[sl], precision, dev)

    r = resident(form)
    exc = torch.empty((), dtype=torch.float64, device=dev)
    vxc = torch.empty((2, args.n_ao, args.n_ao), dtype=torch.float64, device=dev)

    def step(res=r):
        res.xc_energy_and_grads(rdm1, fn, None, True, exc, vxc)
        if world > 1:
            from graddft_gb300 import sharding

            sharding.allreduce_sum([exc, vxc])

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    r.status()
    lib.gdft_profile_reset()
    lib.gdft_profile_enable(1)
    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        barrier()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
    lib.gdft_profile_enable(0)
    r.status()
    ms = e0.elapsed_time(e1)
    import ctypes

    stage = {}
    for name, sid in (("density", _lib.STAGE_DENSITY), ("point", _lib.STAGE_POINT), ("vxc", _lib.STAGE_VXC),
                      ("reduce", _lib.STAGE_REDUCE)):
        t, n = ctypes.c_double(), ctypes.c_int64()
        _lib.check(lib.gdft_profile_read(sid, ctypes.byref(t), ctypes.byref(n)))
        stage[name] = (t.value, n.value)
    # Kernels per step of the library's XC call (the stage timers count regions, some of which hold
    # several kernels): mixed pack_rdm1, dens_tc, xc_point, energy_reduce, build_q, tcg3, vxc_q_reduce;
    # FP64 dens_f64, xc_point, energy_reduce, vxc_f64, vxc_reduce.
    launches = (7 if form == "tf32x3" else 5) * args.steps
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t)
    ms_step = ms / args.steps
    value = world * args.n_grid / (ms_step * 1e-3)
    e_mixed, v_mixed = exc.clone(), vxc.clone()

    # e2e: the same call with host buffers (pinned rdm1 in, E and V out) per step.
    h_rdm1 = rdm1.cpu().pin_memory()
    h_v = torch.empty(vxc.shape, dtype=torch.float64).pin_memory()
    h_e = torch.empty((), dtype=torch.float64).pin_memory()
    d_rdm1 = torch.empty_like(rdm1)

    def e2e_step():
        d_rdm1.copy_(h_rdm1, non_blocking=True)
        r.xc_energy_and_grads(d_rdm1, fn, None, True, exc, vxc)
        h_v.copy_(vxc, non_blocking=True)
        h_e.copy_(exc, non_blocking=True)

    for _ in range(args.warmup):
        e2e_step()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        e2e_step()
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / args.steps
    e2e = {"value": world * args.n_grid / (e2e_ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": rdm1.numel() * 8,
           "d2h_bytes_per_step": vxc.numel() * 8 + 8,
           "note": "molecule (grid, AO tables) resident as after to_device_arrays; rdm1 in, E_xc and V_xc out"}

    # The other form on the same full workload: FP64 rate and the accuracy of the mixed form, over
    # args.seeds seeded workloads (the first is the timed one); the worst case is reported.
    other = {}
    if form == "tf32x3" and not args.no_fp64:
        del r
        torch.cuda.empty_cache()
        per_seed, ms64 = [], None
        for seed in range(SEED, SEED + max(1, args.seeds)):
            wl_s, sl = (wl, mine) if seed == SEED else workload(seed)
            d_s = torch.as_tensor(wl_s.rdm1, device=dev)
            if seed == SEED:
                e_m, v_m = e_mixed, v_mixed
            else:
                r_m = resident("tf32x3", wl_s, sl)
                r_m.xc_energy_and_grads(d_s, fn, None, True, exc, vxc)
                if world > 1:
                    sharding.allreduce_sum([exc, vxc])
                r_m.status()
                e_m, v_m = exc.clone(), vxc.clone()
                del r_m
                torch.cuda.empty_cache()
            r64 = resident("fp64", wl_s, sl)
            r64.xc_energy_and_grads(d_s, fn, None, True, exc, vxc)  # warm
            torch.cuda.synchronize()
            e0.record(stream)
            r64.xc_energy_and_grads(d_s, fn, None, True, exc, vxc)
            e1.record(stream)
            torch.cuda.synchronize()
            if world > 1:
                sharding.allreduce_sum([exc, vxc])
            r64.status()
            if seed == SEED:
                ms64 = e0.elapsed_time(e1)
            per_seed.append({"seed": seed, "E_xc": float(exc), "abs_dE": abs(float(e_m) - float(exc)),
                             "max_abs_V": float(vxc.abs().max()), "max_abs_dV": float((v_m - vxc).abs().max())})
            del r64
            torch.cuda.empty_cache()
        if world > 1:  # the FP64 step above was one rank's slice; the rate is per point
            import torch.distributed as dist

            t = torch.tensor([ms64], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms64 = float(t)
        worst = {"abs_dE": max(a["abs_dE"] for a in per_seed), "max_abs_dV": max(a["max_abs_dV"] for a in per_seed)}
        other = {
            "fp64_form_value": world * args.n_grid / (ms64 * 1e-3), "fp64_form_ms_per_step": ms64,
            "mixed_over_fp64": (world * args.n_grid / (ms_step * 1e-3)) / (world * args.n_grid / (ms64 * 1e-3)),
            "accuracy_vs_fp64": {**per_seed[0], "worst_over_seeds": worst, "seeds": per_seed,
                                 "target": {"abs_dE": 1e-6, "max_abs_dV": 1e-7}},
        }

    # Roofline of the dominant kernel.
    hbm, bf16, src = _peaks()
    dom = max(("density", "vxc"), key=lambda k: stage[k][0])
    t_dom, n_dom = stage[dom]
    flops_launch = 16.0 * args.n_grid * args.n_ao ** 2  # 2 spins x 4 planes x 2 N n^2 per contraction
    achieved = flops_launch / (t_dom / n_dom * 1e-3) / 1e12
    if form == "fp64":
        peak, bound, peak_src = 1.25, "fp64", "nominal GB300 FP64 rate (no measured FP64 peak)"
    else:
        peak, bound, peak_src = bf16, "tensor", f"{src} bf16 dense (the TF32 pipe nominally runs at half of it)"
    traffic = None
    if form == "tf32x3":
        traffic = _profiled_traffic({"density": "dens_tc", "vxc": "tcg_vxc"}[dom], args.n_grid, args.n_ao)
    roof = {"bound": bound, "kernel": f"{dom}_{form}", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak, "peak_source": peak_src, "traffic": traffic,
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of a 65,536-point capture "
                              "(profiles/), scaled by grid points" if traffic else None,
            "flops_per_launch": flops_launch,
            # TF32 products per term: three in the density, six in the V_xc GEMM.
            "executed_flops_per_launch": flops_launch * ((3 if dom == "density" else 6) if form == "tf32x3" else 1),
            # The same stage measured as the tensor work it executes, against the
            # TF32 rate (nominally half the dense BF16 one).
            "executed_tflops": (flops_launch * ((3 if dom == "density" else 6) if form == "tf32x3" else 1)
                                / (t_dom / n_dom * 1e-3) / 1e12),
            "executed_frac_of_tf32": ((flops_launch * (3 if dom == "density" else 6) / (t_dom / n_dom * 1e-3) / 1e12)
                                      / (peak / 2) if form == "tf32x3" else None),
            "stage_ms_per_step": {k: v[0] / args.steps for k, v in stage.items()}}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if form == "fp64" else "tf32x3",
        "data": "synthetic (seeded Gaussian basis evaluated on the device)",
        "config": {"workload": _workload(args.n_grid, args.n_ao), "n_ao": args.n_ao, "n_grid": args.n_grid, "form": form,
                   "functional": "B88+LYP", "l2": "inputs larger than L2 (AO tables "
                                                 f"{5 * args.n_grid * args.n_ao * 8 / 2**30:.1f} GiB per layout)"},
        "roofline": roof, "e2e": e2e, "gpu_launches": launches, "clocks": clk.summary(), **other,
    }
    if rank == 0 and not args.no_cpu:
        # The CPU baseline is the reference arm itself, run in a fresh interpreter (no CUDA context, no
        # GPU-side threads), so the two report one measurement protocol: median of 5 calls after 2 warm-ups.
        import tempfile

        dump = os.path.join(tempfile.mkdtemp(), "oracle_sample.npz")
        env = {k: v for k, v in os.environ.items() if k not in ("RANK", "LOCAL_RANK", "WORLD_SIZE")}
        ref = subprocess.run([sys.executable, os.path.abspath(__file__), "--impl", "reference", "--steps", "5",
                              "--warmup", "2", "--cpu-sample", str(args.cpu_sample), "--n-grid", str(args.n_grid),
                              "--n-ao", str(args.n_ao), "--dump", dump], capture_output=True, text=True, env=env,
                             check=True)
        ref_line = json.loads(ref.stdout.strip().splitlines()[-1])
        line["cpu_baseline"] = {**ref_line["cpu_baseline"], "sample": ref_line["cpu_baseline"]["sample"] +
                                " (the --impl reference arm, run as a child process)"}
        got = np.load(dump)
        e_o, v_o = float(got["exc"]), got["vxc"]
        wl_c = synthetic.make_workload(args.n_grid, args.n_ao, N_OCC, SEED)
        idx = slice(0, args.cpu_sample)
        # Both forms against the oracle on that sample (the same points, basis and D at the full n_ao).
        vs_oracle = {"points": args.cpu_sample}
        for prec in ("fp64", form) if form != "fp64" else ("fp64",):
            r_s = engine.Resident.from_basis(wl_c.basis.packed(), wl_c.coords[idx], wl_c.weights[idx], prec, dev)
            e_g, v_g = r_s.xc_energy_and_grads(torch.as_tensor(wl_c.rdm1, device=dev), fn)
            r_s.status()
            vs_oracle[prec] = {"abs_dE": abs(float(e_g) - e_o), "rel_dE": abs(float(e_g) - e_o) / abs(e_o),
                               "max_abs_dV": float(np.max(np.abs(v_g.cpu().numpy() - v_o))),
                               "rel_dV": float(np.max(np.abs(v_g.cpu().numpy() - v_o)) / np.max(np.abs(v_o)))}
            del r_s
        line["accuracy_vs_oracle_sample"] = vs_oracle
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
