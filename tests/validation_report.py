"""Full-size validation runs (not collected by pytest; run on a GPU machine):

  python tests/validation_report.py precision   # 48^3x96, eps 0.3: FP32 (c64, r12) per-observable
                                                 # errors vs FP64 GPU and vs the FP64 oracle
  python tests/validation_report.py fd          # 32^3x64, eps 0.3: gradients vs central finite
                                                 # differences along random su(3) directions and
                                                 # vs the oracle's analytic staple force
  python tests/validation_report.py flow        # 32^3x64, eps 0.3: RK3 Wilson flow to t = 2.0
                                                 # with B^2 every 0.1, c128 and c64

Each prints a markdown report on stdout.
"""
import os
import sys
import time

import numpy as np
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from flue_gb300 import flow, forces, generate, gluonCalc as G, precision  # noqa: E402
from flue_gb300.field import GaugeField  # noqa: E402


def md_table(rows, head):
    out = ["| " + " | ".join(head) + " |", "|" + "---|" * len(head)]
    out += ["| " + " | ".join(str(c) for c in r) + " |" for r in rows]
    return "\n".join(out)


def run_precision(dims=(96, 48, 48, 48), eps=0.3, seed=3):
    t0 = time.time()
    f = generate.random_field_philox(dims, eps, seed, prec="c128")
    rep = precision.precision_report(f)
    # tie the FP64 GPU values to the oracle on the same field
    U = f.to_numpy()
    oracle.build()
    chk = {}
    s_all, n_all = oracle.genplaquette(U, 1, 4, 4, parallel=True)
    chk["plaquette sum (1,4,4)"] = (G.plaquette(f, 1, 4, 4)[0], s_all)
    chk["polyakov sum Re Tr"] = (G.polyakov(f)[0], oracle.polyakov(U)[0])
    t1 = time.time()
    chk["B^2 (magnetic)"] = (G.magnetic(f), oracle.magnetic(U, parallel=True))
    t_or = time.time() - t1
    b2_32 = {p: G.magnetic(GaugeField.from_array(f, prec=p)) for p in ("c64", "r12")}
    print(f"# Precision report: {dims[1]}^3x{dims[0]}, eps {eps}, seed {seed} (GPU Philox field)\n")
    print("Command: `python tests/validation_report.py precision`\n")
    print("FP64 GPU vs the FP64 oracle on the same field:\n")
    rows = [[k, f"{a:.15e}", f"{b:.15e}", f"{abs(a - b) / abs(b):.2e}"] for k, (a, b) in chk.items()]
    print(md_table(rows, ["observable", "GPU FP64", "oracle (FP64, OpenMP)", "rel diff"]))
    ob = chk["B^2 (magnetic)"][1]
    print(f"\nFP32 B^2 against the oracle: c64 {abs(b2_32['c64'] - ob) / ob:.2e}, r12 {abs(b2_32['r12'] - ob) / ob:.2e} "
          f"(oracle B^2 took {t_or:.1f} s on {oracle.num_threads()} threads)\n")
    keys = [k for k in rep["c64"].keys()]
    rows = [[k, f"{rep['c64'][k]:.2e}", f"{rep['r12'][k]:.2e}"] for k in keys]
    print("FP32 error against FP64 (same field; relative unless noted):\n")
    print(md_table(rows, ["observable", "c64 (FP32, 18 reals)", "r12 (FP32, reconstruct-12)"]))
    print(f"\nFP64 values: {rep['fp64_values']}\n\nwall time {time.time() - t0:.0f} s")


def _perturb(f64: GaugeField, X: torch.Tensor, h: float) -> GaugeField:
    U = f64.to_tensor()  # [t,x,y,z,mu,a,b] view
    E = torch.linalg.matrix_exp(h * X)
    return GaugeField.from_array(torch.matmul(E, U))


def run_fd(dims=(64, 32, 32, 32), eps=0.3, seed=4, ndir=64, h=1e-4):
    t0 = time.time()
    f = generate.random_field_philox(dims, eps, seed, prec="c128")
    print(f"# Gradient checks: {dims[1]}^3x{dims[0]}, eps {eps}, FP64, central FD h = {h}, {ndir} random su(3) directions\n")
    print("Command: `python tests/validation_report.py fd`\n")
    lam = torch.as_tensor(generate.GELL_MANN, device="cuda")
    rows = []
    for name, fn in (("B^2", lambda F: forces.magnetic_force(F, with_force=False)[0]),
                     ("5-loop energy (6 planes)", lambda F: forces.loop5_energy_force(F)[0]),
                     ("plaquette action", lambda F: forces.plaquette_force(F)[0])):
        if name == "B^2":
            _, g = forces.magnetic_force(f)
        elif name.startswith("5-loop"):
            _, g = forces.loop5_energy_force(f)
        else:
            _, g = forces.plaquette_force(f)
        worst, errs = 0.0, []
        nd = ndir if name == "B^2" else max(8, ndir // 8)
        for k in range(nd):
            gen = torch.Generator(device="cuda")
            gen.manual_seed(1000 + k)
            x = torch.randn(tuple(dims) + (4, 8), generator=gen, device="cuda", dtype=torch.float64)
            X = 0.5j * torch.einsum("...a,aij->...ij", x.to(torch.complex128), lam)
            fp = fn(_perturb(f, X, h))
            fm = fn(_perturb(f, X, -h))
            fd = (fp - fm) / (2 * h)
            an = float(-2.0 * torch.einsum("...ij,...ji->", X, g).real)
            errs.append(abs(an - fd) / abs(fd))
        rows.append([name, nd, f"{np.median(errs):.2e}", f"{max(errs):.2e}"])
    print(md_table(rows, ["observable", "directions", "median rel(analytic - FD)", "max"]))
    # analytic staple force vs the oracle
    oracle.build()
    U = f.to_numpy()
    go = oracle.plaquette_staple_force(U)
    _, gp = forces.plaquette_force(f)
    d = float(np.abs(gp.cpu().numpy() - go).max())
    print(f"\nPlaquette-action gradient vs the oracle's analytic staple force: max |diff| = {d:.2e} "
          f"(max |G| = {float(np.abs(go).max()):.3f})\n\nwall time {time.time() - t0:.0f} s")


def run_flow(dims=(64, 32, 32, 32), eps=0.3, seed=5, step=0.01, tmax=2.0, every=0.1):
    t0 = time.time()
    f = generate.random_field_philox(dims, eps, seed, prec="c128")
    print(f"# Wilson flow: {dims[1]}^3x{dims[0]}, eps {eps}, RK3 step {step} to t = {tmax}, B^2 every {every}\n")
    print("Command: `python tests/validation_report.py flow`\n")
    res = {}
    times = {}
    for p in ("c128", "c64"):
        torch.cuda.synchronize()
        t1 = time.time()
        _, recs = flow.wilson_flow(GaugeField.from_array(f, prec=p), eps=step, tmax=tmax, measure_every=every)
        torch.cuda.synchronize()
        times[p] = time.time() - t1
        res[p] = recs
    rows = []
    for a, b in zip(res["c128"], res["c64"]):
        rows.append([f"{a['t']:.2f}", f"{a['plaq']:.12f}", f"{a['b2']:.10e}", f"{b['b2']:.10e}",
                     f"{abs(a['b2'] - b['b2']) / a['b2']:.1e}"])
    print(md_table(rows, ["t", "<Re Tr P>/3 (FP64)", "B^2 FP64", "B^2 FP32 (c64)", "rel diff"]))
    print(f"\nflow wall time: FP64 {times['c128']:.1f} s, FP32 {times['c64']:.1f} s "
          f"({int(round(tmax / step))} RK3 steps + {len(rows)} B^2 measurements each); total {time.time() - t0:.0f} s")


if __name__ == "__main__":
    what = sys.argv[1] if len(sys.argv) > 1 else "precision"
    {"precision": run_precision, "fd": run_fd, "flow": run_flow}[what]()
