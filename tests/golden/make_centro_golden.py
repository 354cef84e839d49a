"""Generate tests/golden/centro_reference.json from the reference itself.

Runs the reference visualiser's computeCentrosymmetry
(src-viz/AtomVisualize.c:399-672), compiled from its own text without the
graphics by oracle/Makefile (oracle/_ref/libcomdref_centro{,_approx}.so),
on the inputs `centro_cases` builds with this library's reference-identical
host setup (create_fcc_lattice, the seeded displacements, the clsman
reader).  For each case and each pairing rule (exact; APPROX_CENTROSYM) it
records a sha256 of the per-atom values in id order, their sum, the first
ids' values and the routine's minCentro / maxCentro, so the oracle and the
GPU kernel can be checked against the reference where its sources are
absent.

Usage: python tests/golden/make_centro_golden.py   (needs oracle/_ref built)
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import comd_gb300 as cg  # noqa: E402
from comd_gb300.abi import occupied_mask, slot_views  # noqa: E402
from oracle import ref_centro  # noqa: E402

NIDS = 12

# name -> how the input is built (read by centro_case).  Displacements are
# the seeded uniform kind (integer hashing and one multiply per component),
# so every host builds the same positions bit for bit; the Gaussian kind
# goes through the host's log and cos.
CASES = {
    "cu6_perfect": {"kind": "fcc", "pot": "cu", "n": 6, "defgrad": 1.0, "bf": 1.0},
    "cu8_disp": {"kind": "fcc", "pot": "cu", "n": 8, "defgrad": 1.0, "bf": 1.0,
                 "seed": [21, 1, 0.12, 0.0, 63.55]},
    "cu8_stretch_bf12_disp": {"kind": "fcc", "pot": "cu", "n": 8, "defgrad": 1.05, "bf": 1.2,
                              "seed": [5, 1, 0.08, 0.0, 63.55]},
    "cu3_two_box_grid_disp": {"kind": "fcc", "pot": "cu", "n": 3, "defgrad": 1.0, "bf": 1.0,
                              "seed": [4, 1, 0.12, 0.0, 63.55]},
    "ag8k_file": {"kind": "clsman", "pot": "ag", "file": "8k.inp.gz", "bf": 1.0},
}


def centro_case(spec):
    """(host simflat_t, potential) for a case spec; the caller frees both"""
    pot = cg.eam_potential(spec["pot"])
    if spec["kind"] == "fcc":
        n = spec["n"]
        s = cg.fcc(n, n, n, pot.ptr.contents.lat, spec["defgrad"], spec["bf"], pot)
        if "seed" in spec:
            cg.seed(s, *spec["seed"])
    else:
        s = cg.read_clsman(os.path.join(cg.DATA_DIR, spec["file"]), pot, spec["bf"], -1)
    return s, pot


def by_id(s, per_slot):
    """the occupied slots' values in atom-id order"""
    v = slot_views(s)
    m = occupied_mask(s)
    return per_slot[m][np.argsort(v["id"][m], kind="stable")]


def digest(values):
    return hashlib.sha256(np.ascontiguousarray(values, dtype="<f8").tobytes()).hexdigest()


def layout_digest(s):
    v = slot_views(s)
    m = occupied_mask(s)
    h = hashlib.sha256()
    h.update(v["natoms"].astype("<i4").tobytes())
    h.update(v["id"][m].astype("<i4").tobytes())
    h.update(np.ascontiguousarray(v["r"][m], dtype="<f8").tobytes())
    return h.hexdigest()


def main():
    refs = {False: ref_centro(False), True: ref_centro(True)}
    if refs[False] is None or refs[True] is None:
        sys.exit("oracle/_ref holds no centrosymmetry build (run make -C oracle REF=<reference>)")
    fx = {"generator": "tests/golden/make_centro_golden.py (reference AtomVisualize::"
                       "computeCentrosymmetry via oracle/_ref)", "cases": {}}
    for name, spec in CASES.items():
        s, _pot = centro_case(spec)
        try:
            out = {"spec": spec, "ntot": s.contents.ntot, "nbx": list(s.contents.nbx),
                   "input": layout_digest(s)}
            for approx in (False, True):
                c, lo, hi = refs[approx].centro(s)
                vals = by_id(s, c)
                out["approx" if approx else "exact"] = {
                    "sha256": digest(vals), "sum": float(vals.sum()),
                    "first": vals[:NIDS].tolist(), "min_centro": lo, "max_centro": hi}
            fx["cases"][name] = out
        finally:
            cg.free_host(s)
    path = os.path.join(HERE, "centro_reference.json")
    with open(path, "w") as f:
        json.dump(fx, f, indent=1)
    print("wrote", path)


if __name__ == "__main__":
    main()
