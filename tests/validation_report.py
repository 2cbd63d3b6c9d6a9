"""Full-size validation runs (not collected by pytest; run on a GPU machine):

  python tests/validation_report.py precision   # 48^3x96, eps 0.3: FP32 (c64, r12) per-observable
                                                 # errors vs FP64 GPU and vs the FP64 oracle
  python tests/validation_report.py fd          # 32^3x64, eps 0.3: gradients vs central finite
                                                 # differences along random su(3) directions and
                                                 # vs the oracle's analytic staple force
  python tests/validation_report.py flow        # 32^3x64, eps 0.3: RK3 Wilson flow to t = 2.0
                                                 # with B^2 every 0.1, c128 and c64
  python tests/validation_report.py config1     # 32^3x64, eps 0.1, 0.5 and Haar: every observable
                                                 # (FP64 GPU, FP32 c64 and r12) against the oracle

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


def _cmp_scalar(a, b, per=None):
    """relative difference, or absolute per unit when the sum can cancel"""
    if per:
        return abs(a - b) / per
    return abs(a - b) / max(abs(b), 1e-300)


def _cmp_field(a, b):
    """max |a - b| / max |b| over a matrix field"""
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    return float(np.abs(a.astype(np.complex128) - b).max() / np.abs(b).max())


def _config1_field(dims, eps, seed):
    if eps == "haar":
        U = generate.haar_field(dims, seed)
        return GaugeField.from_array(U), U
    f = generate.random_field(dims, eps, seed, device="cuda")
    return f, f.to_numpy()


def run_config1(dims=(64, 32, 32, 32), cases=((0.1, 21), (0.5, 22), ("haar", 23))):
    """Every observable of the path at 32^3 x 64 against the oracle, on a
    near-cold (eps 0.1), a rough (eps 0.5) and a Haar-random field: FP64 GPU,
    FP32 complex64 and FP32 reconstruct-12."""
    t_all = time.time()
    oracle.build()
    paths = ([1, 2, -1, -2], [2, 2, 3, -4, -2, 1, 1, -3], [3, 3, 3, 2, -3, -3, -3, -2])
    b2_planes = ((3, 2), (2, 4), (4, 3))
    print(f"# Parity at {dims[1]}^3x{dims[0]}: every observable against the FP64 oracle\n")
    print("Command: `python tests/validation_report.py config1`\n")
    print("Fields: links exp(i eps H) (H from PCG64(seed) Gell-Mann coefficients, exponentials on the GPU, then "
          "FixSU3Matrix) at eps 0.1 and 0.5, and a Haar-random field (host QR of complex Gaussians). "
          "Differences: relative for sums that do not cancel; for sums that can (Haar plaquettes and Polyakov "
          "loops) the absolute difference per plaquette / per spatial site; max |diff| / max |oracle| for "
          "matrix fields (genericPath at every site, clover and 5-loop F); absolute for W(R,T) and u0. "
          f"Oracle: `oracle/flue_oracle.c`, {oracle.num_threads()} OpenMP threads.\n")
    for eps, seed in cases:
        t0 = time.time()
        f, U = _config1_field(dims, eps, seed)
        fields = {"c128": f, "c64": GaugeField.from_array(f, prec="c64"), "r12": GaugeField.from_array(f, prec="r12")}
        rows = {}
        haar = eps == "haar"
        # plaquettes
        for name, r in (("plaquette all (1,4,4)", (1, 4, 4)), ("plaquette spatial (2,4,4)", (2, 4, 4)),
                        ("plaquette temporal (1,1,4)", (1, 1, 4))):
            so, no = oracle.genplaquette(U, *r, parallel=True)
            rows[name] = (f"{so / no / 3:.12f}", [_cmp_scalar(G.plaquette(fields[p], *r)[0], so, no if haar else None)
                                                  for p in fields])
        so, no = oracle.polyakov(U)
        rows["Polyakov sum Re Tr"] = (f"{so:.6e}", [_cmp_scalar(G.polyakov(fields[p])[0], so, no) for p in fields])
        for path in paths:
            go = oracle.genericpath_all(U, path)
            rows[f"genericPath {path}"] = ("(field)", [_cmp_field(G.genericpath_all(fields[p], path), go) for p in fields])
            del go
        tab_o = np.array([[oracle.wmunu(U, 2, 3, r + 1, t + 1, parallel=True) for t in range(8)] for r in range(8)])
        errs = []
        for p in fields:
            tab = G.wmunu_table(fields[p], 2, 3, 8, 8)
            tab = tab.detach().cpu().numpy() if isinstance(tab, torch.Tensor) else np.asarray(tab)
            errs.append(float(np.abs(tab - tab_o).max()))
        rows["W_xy(R,T), R,T = 1..8 (max abs)"] = (f"W(1,1) {tab_o[0, 0]:.10f}, W(8,8) {tab_o[7, 7]:.3e}", errs)
        for mu, nu in b2_planes:
            co = oracle.cloverloopmunucoord(U, mu, nu)
            rows[f"clover F({mu},{nu})"] = (f"max {np.abs(co).max():.4f}",
                                            [_cmp_field(G.cloverloopmunucoord(fields[p], mu, nu), co) for p in fields])
            del co
            qo = oracle.loop5munucoord(U, mu, nu)
            rows[f"5-loop F({mu},{nu})"] = (f"max {np.abs(qo).max():.4f}",
                                            [_cmp_field(G.loop5munucoord(fields[p], mu, nu), qo) for p in fields])
            del qo
        bo = oracle.magnetic(U, parallel=True)
        rows["B^2 (magnetic)"] = (f"{bo:.12e}", [_cmp_scalar(G.magnetic(fields[p]), bo) for p in fields])
        gt = generate.random_gauge_transform(dims, seed + 100)
        uo = oracle.uzerobar(U, gt)
        errs = []
        for p in fields:
            a = np.asarray(G.uzerobar(fields[p], gt))
            ok = ~np.isnan(uo)
            assert np.array_equal(np.isnan(a), np.isnan(uo))
            errs.append(float(np.abs(a[ok] - uo[ok]).max()) if ok.any() else 0.0)
        rows["u0 (plaquette all/spatial/temporal, Landau all/spatial/temporal; max abs)"] = (
            " ".join(f"{v:.8f}" for v in uo), errs)
        label = "Haar-random" if haar else f"eps {eps}"
        print(f"## {label} (seed {seed})\n")
        print(md_table([[k, v[0]] + [f"{e:.1e}" for e in v[1]] for k, v in rows.items()],
                       ["observable", "oracle value", "FP64 GPU", "FP32 c64", "FP32 r12"]))
        worst64 = max(v[1][0] for v in rows.values())
        print(f"\nworst FP64 difference {worst64:.1e}; field built and checked in {time.time() - t0:.0f} s\n")
        del fields, f, U
        torch.cuda.empty_cache()
    print(f"total wall time {time.time() - t_all:.0f} s")


if __name__ == "__main__":
    what = sys.argv[1] if len(sys.argv) > 1 else "precision"
    {"precision": run_precision, "fd": run_fd, "flow": run_flow, "config1": run_config1}[what]()
