"""Generate the golden fixtures of the test-suite.

abelian_kat.json -- analytic known answers.  On an L_T x L_X x L_Y x L_Z
periodic lattice the diagonal SU(3) field
    U_x(t,x,y,z) = diag(e^{-i phi_a y}),
    U_y(t,x,y,z) = diag(e^{+i phi_a L_Y x}) on y = L_Y - 1, else 1,
    U_t = diag(e^{i alpha_a}),  U_z = 1,
with phi_a = 2 pi n_a / (L_X L_Y), sum_a n_a = 0, sum_a alpha_a = 0, has a
constant abelian flux: every a x b rectangle in the (x,y) plane, traversed
x first, equals diag(e^{i a b phi_a}); every other plaquette is 1.  Hence
(reference conventions: sums of Re Tr, no 1/3, directions 1-based)
    plaquette(1,4,4)      = V (15 + sum_a cos phi_a)
    plaquette(2,4,4)      = V (6 + sum_a cos phi_a)
    plaquette(1,1,4)      = 9 V
    polyakov              = NX NY NZ sum_a cos(NT alpha_a)
    wmunu(2,3,R,T)        = sum_a cos(R T phi_a)
    clover F(2,3)         = diag(i sin phi_a)
    5-loop F(2,3)         = diag(i f_a),
        f_a = k1 sin phi_a + k2 sin 4phi_a + k5 sin 9phi_a + k3 sin 2phi_a + k4 sin 3phi_a
    magnetic (B^2)        = sum_a f_a^2
with the 5-loop coefficients of src/wloops.F90:219-224.  The closed forms are
evaluated here in exact-rational / mpmath-free double arithmetic from the
formulas above (no lattice code involved).

oracle_regression.json -- outputs of the C oracle on seeded random fields,
committed so that any later change to the oracle is detected.

Run from the repository root:  python tests/golden/make_golden.py
"""
import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

K5 = 1.0 / 180.0
K1 = 19.0 / 9.0 - 55.0 * K5
K2 = 1.0 / 36.0 - 16.0 * K5
K3 = 64.0 * K5 - 32.0 / 45.0
K4 = 1.0 / 15.0 - 6.0 * K5

KAT_CASES = [
    {"dims": [4, 4, 4, 4], "n": [1, -1, 0], "alpha": [0.3, -0.1, -0.2]},
    {"dims": [6, 4, 5, 3], "n": [2, 1, -3], "alpha": [0.7, 0.2, -0.9]},
    {"dims": [5, 6, 6, 4], "n": [1, 2, -3], "alpha": [1.1, -0.4, -0.7]},
]


def kat_expected(case):
    nt, nx, ny, nz = case["dims"]
    V = nt * nx * ny * nz
    phi = [2 * math.pi * n / (nx * ny) for n in case["n"]]
    alpha = case["alpha"]
    cs = sum(math.cos(p) for p in phi)
    f = [K1 * math.sin(p) + K2 * math.sin(4 * p) + K5 * math.sin(9 * p) + K3 * math.sin(2 * p) + K4 * math.sin(3 * p)
         for p in phi]
    return {
        "plaq_all": V * (15 + cs),
        "plaq_spatial": V * (6 + cs),
        "plaq_temporal": 9.0 * V,
        "polyakov": nx * ny * nz * sum(math.cos(nt * a) for a in alpha),
        "wmunu_23": {f"{r},{t}": sum(math.cos(r * t * p) for p in phi) for r in (1, 2, 3) for t in (1, 2, 3)},
        "clover_diag_im": [math.sin(p) for p in phi],
        "loop5_diag_im": f,
        "magnetic": sum(v * v for v in f),
    }


def abelian_field(case):
    nt, nx, ny, nz = case["dims"]
    phi = np.array([2 * math.pi * n / (nx * ny) for n in case["n"]])
    alpha = np.array(case["alpha"])
    U = np.zeros((nt, nx, ny, nz, 4, 3, 3), dtype=np.complex128)
    t, x, y, z = np.meshgrid(np.arange(nt), np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    for a in range(3):
        U[..., 0, a, a] = np.exp(1j * alpha[a])
        U[..., 1, a, a] = np.exp(-1j * phi[a] * y)
        U[..., 2, a, a] = np.where(y == ny - 1, np.exp(1j * phi[a] * ny * x), 1.0)
        U[..., 3, a, a] = 1.0
    return np.asfortranarray(U)


def regression():
    import oracle
    from flue_gb300 import generate

    out = []
    for dims, eps, seed in (([4, 4, 4, 6], 0.3, 11), ([3, 4, 5, 4], 0.5, 12)):
        U = generate.random_field(dims, eps, seed)
        rec = {"dims": dims, "eps": eps, "seed": seed}
        rec["plaq_all"] = oracle.plaquette(U, 1, 4, 4)[0]
        rec["plaq_spatial"] = oracle.plaquette(U, 2, 4, 4)[0]
        rec["plaq_temporal"] = oracle.plaquette(U, 1, 1, 4)[0]
        rec["polyakov"] = oracle.polyakov(U)[0]
        rec["wmunu_23_2_3"] = oracle.wmunu(U, 2, 3, 2, 3)
        rec["wmunutau_2_14_1_2"] = oracle.wmunutau(U, 2, 1, 4, 1, 2)
        rec["magnetic"] = oracle.magnetic(U)
        f = oracle.loop5munucoord(U, 3, 2)
        rec["loop5_32_site0"] = [[f[0, 0, 0, 0, a, b].real, f[0, 0, 0, 0, a, b].imag] for a in range(3) for b in range(3)]
        rec["loop5_32_sumabs"] = float(np.abs(f).sum())
        c = oracle.cloverloopmunucoord(U, 1, 3)
        rec["clover_13_sumabs"] = float(np.abs(c).sum())
        g = oracle.genericpath(U, [2, 1, 3, 1], [1, 2, -1, 3, -2, -3, 4])
        rec["genericpath"] = [[g[a, b].real, g[a, b].imag] for a in range(3) for b in range(3)]
        out.append(rec)
    return out


def main():
    kats = []
    for case in KAT_CASES:
        kats.append({"case": case, "expected": kat_expected(case)})
    with open(os.path.join(HERE, "abelian_kat.json"), "w") as fh:
        json.dump(kats, fh, indent=1)
    with open(os.path.join(HERE, "oracle_regression.json"), "w") as fh:
        json.dump(regression(), fh, indent=1)


if __name__ == "__main__":
    main()
