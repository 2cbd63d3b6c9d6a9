"""Golden vectors from the reference's own Fortran, run through a translator.

No Fortran compiler is available, so `fortran_subset.py` translates the
reference's `src/constants.f90`, `src/SU3MatrixOps.f90`, `src/wloops.F90`,
the gauge-file readers (`src/gaugeIO/ILDG_bin.f90`,
`src/gaugeIO/openqcdfileio_standalone.f90`, on files written by
`flue_gb300.gaugeIO`) and the analysis helpers (`src/jack.f90`,
`src/gluonAna/momentum.f90`, `src/gluonAna/gpManip.f90`) statement by
statement into Python over numpy (in memory) and runs the
routines as written (serial build: no OpenMP / `do concurrent` macros) on the
fields below.  Their outputs are stored in `reference_fortran.json` with the
recipe of every input, so that the oracle (CPU) and the CUDA library (GPU)
are compared with the reference's own code paths, not only with a
restatement of them.

Inputs: seeded fields of `flue_gb300.generate` (numpy PCG64: `random_field`
= exp(i eps H) links, `haar_field` = Haar-random SU(3)), rebuilt by the
tests from the recipe and checked against the stored checksums; random 3x3
complex matrices drawn from PCG64 and stored as they are.

Run in a container that holds the reference tree (it is read, never
copied):
    python tests/golden/make_reference_golden.py [/path/to/reference]
The config-0 field (8^3 x 16) takes several minutes in the translated
routines.
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from flue_gb300 import generate  # noqa: E402
from tests.golden import fortran_subset  # noqa: E402

OUT = os.path.join(HERE, "reference_fortran.json")
SOURCES = ("src/constants.f90", "src/SU3MatrixOps.f90", "src/wloops.F90", "src/gaugeIO/ILDG_bin.f90")
ANALYSIS_SOURCES = ("src/jack.f90", "src/gluonAna/momentum.f90", "src/gluonAna/gpManip.f90")
# (the file readers are run on their own, in run_readers)
SKIP = ("readgaugefield_ildg", "readgaugetransformation_cola")
READER_SOURCES = ("src/gaugeIO/ILDG_bin.f90", "src/gaugeIO/openqcdfileio_standalone.f90")
# gauge files for the readers: a 4 x 2 x 4 x 2 field (NT, NX, NY, NZ) made
# slightly non-unitary, so that the readers' FixSU3Matrix has work to do
READER_FIELD = {"dims": [4, 2, 4, 2], "eps": 0.3, "seed": 3, "noise": 1e-3, "noise_seed": 1, "plaq": 1.5,
                "transform_seed": 5}


def reader_inputs(recipe):
    """The field and gauge transformation the reader files are written from."""
    dims = tuple(recipe["dims"])
    U = generate.random_field(dims, recipe["eps"], recipe["seed"])
    rng = np.random.Generator(np.random.PCG64(recipe["noise_seed"]))
    U = np.asfortranarray(U + recipe["noise"] * (rng.standard_normal(U.shape) + 1j * rng.standard_normal(U.shape)))
    G = generate.random_gauge_transform(dims, recipe["transform_seed"])
    return U, G


def write_reader_files(recipe, d):
    """ILDG (big-endian, direct records), openQCD (little-endian stream) and
    cola gauge-transformation (big-endian sequential records) files written
    by flue_gb300.gaugeIO's writers."""
    from flue_gb300 import gaugeIO

    U, G = reader_inputs(recipe)
    paths = {"ildg": os.path.join(d, "field.ildg"), "openqcd": os.path.join(d, "field.oqcd"),
             "cola": os.path.join(d, "transform.cola")}
    gaugeIO.write_ildg_be(paths["ildg"], U)
    gaugeIO.write_openqcd(paths["openqcd"], U, plaq=recipe["plaq"])
    gaugeIO.write_gauge_transformation_cola(paths["cola"], G)
    return paths


def field(recipe):
    if recipe["kind"] == "random":
        return generate.random_field(tuple(recipe["dims"]), recipe["eps"], recipe["seed"])
    if recipe["kind"] == "haar":
        return generate.haar_field(tuple(recipe["dims"]), recipe["seed"])
    raise ValueError(recipe["kind"])


def checksum(U):
    """Sum of |U|^2 and a weighted sum that depends on every element's place."""
    w = np.cos(np.arange(U.size, dtype=np.float64) * 0.61803398875).reshape(U.shape, order="F")
    return [float(np.sum(np.abs(U) ** 2)), float(np.sum(w * U.real)), float(np.sum(w * U.imag))]


def cplx(a):
    a = np.asarray(a)
    return [np.real(a).ravel(order="F").tolist(), np.imag(a).ravel(order="F").tolist()]


def field_summary(F):
    """An F field (NT,NX,NY,NZ,3,3): its checksum and the matrices at 12
    sites spread over the lattice (linear site index, time fastest)."""
    V = int(np.prod(F.shape[:4]))
    flat = F.reshape((V, 3, 3), order="F")
    sites = sorted({int(round(k * (V - 1) / 11)) for k in range(12)})
    return {"checksum": checksum(F), "sites": {str(k): cplx(flat[k]) for k in sites}}


# observables per field; "full" adds the clover and 5-loop F fields (their
# checksums and 12 sites each; small lattices only)
CASES = [
    {"name": "random_4x3x4x3", "recipe": {"kind": "random", "dims": [4, 3, 4, 3], "eps": 0.4, "seed": 5},
     "full": True},
    {"name": "haar_3x4x2x3", "recipe": {"kind": "haar", "dims": [3, 4, 2, 3], "seed": 7}, "full": True},
    {"name": "strong_5x2x3x4", "recipe": {"kind": "random", "dims": [5, 2, 3, 4], "eps": 0.9, "seed": 17},
     "full": True},
    {"name": "haar_2x3x3x2", "recipe": {"kind": "haar", "dims": [2, 3, 3, 2], "seed": 19}, "full": True},
    {"name": "config0_8x8x8x16", "recipe": {"kind": "random", "dims": [16, 8, 8, 8], "eps": 0.3, "seed": 1},
     "full": False},
]
# (coordinates taken modulo each lattice's extents)
PATHS = [
    ([1, 1, 1, 1], [1, 2, -1, -2]),
    ([2, 3, 1, 2], [2, 3, -2, -3, 4, 4, -4, -4]),
    ([3, 2, 2, 1], [-1, -3, 2, 1, 3, -2]),
    ([1, 3, 2, 3], [4, 4, 4, 1, -4, -4, -4, -1]),
]
WLOOPS = [(2, 3, 1, 1), (2, 3, 2, 1), (3, 4, 1, 3), (1, 2, 2, 2), (4, 2, 3, 2)]
WLOOPS_TAU = [(1, 2, 3, 1, 2), (2, 3, 4, 2, 2)]
PLANES = [(3, 2), (2, 4), (4, 3), (1, 2)]


def run_case(ns, case, log):
    U = field(case["recipe"])
    NT, NX, NY, NZ = U.shape[:4]
    out = {"recipe": case["recipe"], "checksum": checksum(U)}
    t = time.time()
    plaq = {}
    for rng in ((1, 4, 4), (2, 4, 4), (1, 1, 4)):
        s, n, _ = ns["plaquette"](U, *rng, 0.0, 0, 0.0)
        sg, ng, _ = ns["genplaquette"](U, NT, NX, NY, NZ, *rng, 0.0, 0, 0.0)
        plaq[",".join(map(str, rng))] = {"sum": s, "n": int(n), "gen_sum": sg, "gen_n": int(ng)}
    out["plaquette"] = plaq
    if NT >= 3:  # (the reference's loop leaves its product undefined for NT < 3)
        s, n, _ = ns["polyakov"](U, 0.0, 0, 0.0)
        out["polyakov"] = {"sum": s, "n": int(n)}
    out["genericpath"] = []
    for c, p in PATHS:
        c = [(ci - 1) % n + 1 for ci, n in zip(c, (NT, NX, NY, NZ))]
        out["genericpath"].append({"coord": c, "path": p,
                                   "matrix": cplx(ns["genericpath"](U, np.array(c), np.array(p)))})
    out["wmunu"] = [{"args": list(a), "value": ns["wmunu"](U, *a)} for a in WLOOPS]
    out["wmunutau"] = [{"args": list(a), "value": ns["wmunutau"](U, *a)} for a in WLOOPS_TAU]
    log(f"  {case['name']}: plaquette, polyakov, paths, loops {time.time() - t:.1f} s")
    if case["full"]:
        out["clover"] = [dict(plane=list(pl), **field_summary(ns["cloverloopmunucoord"](U, NT, NX, NY, NZ, *pl)))
                         for pl in PLANES[:2]]
        out["loop5"] = [dict(plane=list(pl), **field_summary(ns["loop5munucoord"](U, NT, NX, NY, NZ, *pl)))
                        for pl in PLANES]
        log(f"  {case['name']}: clover and 5-loop F {time.time() - t:.1f} s")
    out["magnetic"] = ns["magnetic"](U, NT, NX, NY, NZ)
    log(f"  {case['name']}: magnetic {time.time() - t:.1f} s")
    return out


def run_analysis(ref_root, log):
    """Jackknife (src/jack.f90), get_qhat (src/gluonAna/momentum.f90),
    Q_Average and cone_cut (src/gluonAna/gpManip.f90) on seeded inputs."""
    tr = fortran_subset.Translator()
    for rel in ("src/constants.f90",) + ANALYSIS_SOURCES:
        with open(os.path.join(ref_root, rel)) as f:
            tr.add_source(f.read())
    ns = tr.build()
    np.seterr(invalid="ignore")  # (ACOS of a rounding-level 1+ gives NaN, as in Fortran)
    rng = np.random.Generator(np.random.PCG64(23))
    data = rng.standard_normal(9) + 2.0
    n = data.size
    z = np.zeros(n)
    out = {"data": data.tolist(),
           "complement0": ns["complement0"](0.0, data)[0],
           "complement1": ns["complement1"](n, z, data)[0].tolist(),
           "complement2": {"icon": 3, "value": ns["complement2"](n, z, data, 3)[0].tolist()},
           "complement3": {"icon": 2, "jcon": 7, "value": ns["complement3"](n, z, data, 2, 7)[0].tolist()}}
    c = np.concatenate([[out["complement0"]], out["complement1"]])
    err, bias = ns["jackknife_wp"](n, c, 0.0, 0.0)
    out["jackknife"] = {"c": c.tolist(), "err": err, "bias": bias}
    coords = [[0.0, 1.0, 2.0, 3.0], [3.0, -1.0, 0.0, 2.0], [1.5, 2.5, -2.0, 0.5]]
    out["get_qhat"] = [{"coord": cd, "shape": [8, 4, 6, 4], "a": a,
                        "qhat": ns["get_qhat"](np.array(cd), np.array([8, 4, 6, 4]), np.zeros(4), a)[0].tolist()}
                       for cd in coords for a in (1.0, 0.7)]
    q = np.sort(rng.uniform(0.05, 3.0, 40))
    D = rng.uniform(0.5, 2.0, 40)
    out["q_average"] = {"q": q.tolist(), "D": D.tolist(), "runs": []}
    for qs in (4, 7):
        dout, qout, qcount = ns["q_average"](40, q, D, qs, np.zeros(41), np.zeros(41), 0)
        out["q_average"]["runs"].append({"q_slices": qs, "dout": dout.tolist(), "qout": qout.tolist(),
                                         "qcount": int(qcount)})
    # momenta of a 4^4 lattice (q^ of the index grid, indices above N/2 negative)
    Q = generate_momenta((4, 4, 4, 4))
    NQ = Q.shape[0]
    Dq = rng.uniform(0.5, 2.0, NQ)
    D4 = rng.uniform(0.5, 2.0, NQ)
    out["cone_cut"] = {"lattice": [4, 4, 4, 4], "D": Dq.tolist(), "D4": D4.tolist(), "runs": []}
    for radius, opt in ((1, (None, None, None, None)), (2, (0.6, 1.3, 1.0, 3.0)), (1, (None, 2.0, None, 0.5))):
        qo, do, d4o, cnt = ns["cone_cut"](NQ, radius, Q, Dq, D4, 4, 4, *opt, np.zeros((NQ, 4)), np.zeros(NQ),
                                          np.zeros(NQ), 0)
        out["cone_cut"]["runs"].append({"radius": radius, "angle_xi_ircut_irradius": list(opt),
                                        "qcount": int(cnt), "qout": qo[:cnt].ravel(order="F").tolist(),
                                        "dout": do[:cnt].tolist(), "d4out": d4o[:cnt].tolist()})
    log("  analysis helpers")
    return out


def run_readers(ref_root, log):
    """The reference's gauge-file readers on files of the three formats."""
    import tempfile

    tr = fortran_subset.Translator()
    for rel in ("src/constants.f90",) + READER_SOURCES:
        with open(os.path.join(ref_root, rel)) as f:
            tr.add_source(f.read())
    ns = tr.build()
    nt, nx, ny, nz = READER_FIELD["dims"]
    with tempfile.TemporaryDirectory() as d:
        paths = write_reader_files(READER_FIELD, d)
        out = {"recipe": READER_FIELD,
               "ildg": field_summary7(ns["readgaugefield_ildg"](paths["ildg"], nx, ny, nz, nt)),
               "openqcd": field_summary7(ns["readgaugefield_openqcd"](paths["openqcd"], nx, ny, nz, nt)),
               "cola": field_summary(ns["readgaugetransformation_cola"](paths["cola"], nx, ny, nz, nt))}
    log("  gauge-file readers")
    return out


def field_summary7(U):
    """A gauge field (NT,NX,NY,NZ,4,3,3): checksum and 12 links."""
    V = int(np.prod(U.shape[:4]))
    flat = U.reshape((V * 4, 3, 3), order="F")
    links = sorted({int(round(k * (4 * V - 1) / 11)) for k in range(12)})
    return {"checksum": checksum(U), "links": {str(k): cplx(flat[k]) for k in links}}


def generate_momenta(dims):
    """q^_mu = 2 pi n_mu / N_mu over the index grid, n_mu > N_mu/2 taken as
    n_mu - N_mu; rows in Fortran order of (t, x, y, z)."""
    axes = [np.where(np.arange(n) > n // 2, np.arange(n) - n, np.arange(n)) for n in dims]
    grid = np.stack(np.meshgrid(*axes, indexing="ij"), axis=-1).astype(np.float64)
    q = 2.0 * np.pi * grid / np.asarray(dims, dtype=np.float64)
    return q.transpose(3, 2, 1, 0, 4).reshape(-1, 4)


def main(ref_root):
    tr = fortran_subset.Translator()
    for rel in SOURCES:
        with open(os.path.join(ref_root, rel)) as f:
            tr.add_source(f.read())
    ns = tr.build(only={n for n in tr.procs if n not in SKIP})

    def log(msg):
        print(msg, flush=True)

    rng = np.random.Generator(np.random.PCG64(11))
    mats = [(rng.standard_normal((3, 3)) + 1j * rng.standard_normal((3, 3))) for _ in range(4)]
    zero33 = np.zeros((3, 3), dtype=np.complex128)
    alg = {
        "matrices": [cplx(m) for m in mats],
        "multiplymatmat": cplx(ns["multiplymatmat"](zero33, mats[0], mats[1])[0]),
        "multiplymatdagmatdag": cplx(ns["multiplymatdagmatdag"](zero33, mats[2], mats[3])[0]),
        "realtracemultmatmat": ns["realtracemultmatmat"](0.0, mats[0], mats[3])[0],
        "tracelessconjgsubtract": cplx(ns["tracelessconjgsubtract"](zero33, mats[1], mats[2])[0]),
        "colourdecomp": cplx(ns["colourdecomp"](np.zeros(8, dtype=np.complex128), mats[3])[0]),
    }
    # FixSU3Matrix (re-unitarisation of a stored link): raw random matrices
    # and Haar SU(3) matrices with a 1e-3 perturbation
    haar = generate.haar_field((1, 1, 1, 1), 3)[0, 0, 0, 0]
    fix_in = mats[:2] + [haar[k] + 1e-3 * (rng.standard_normal((3, 3)) + 1j * rng.standard_normal((3, 3)))
                         for k in range(3)]
    alg["fixsu3matrix"] = {"in": [cplx(m) for m in fix_in],
                           "out": [cplx(ns["fixsu3matrix"](m.copy())[0]) for m in fix_in]}
    res = {"sources": list(SOURCES) + list(ANALYSIS_SOURCES) + list(READER_SOURCES), "algebra": alg,
           "analysis": run_analysis(ref_root, log), "readers": run_readers(ref_root, log), "fields": {}}
    for case in CASES:
        res["fields"][case["name"]] = run_case(ns, case, log)
    with open(OUT, "w") as f:
        json.dump(res, f, separators=(",", ":"))
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
