"""Generate tests/golden/reference_fixtures.json from the reference itself.

Runs the reference CoMD src-flat, compiled from its own sources into
oracle/_ref by oracle/Makefile (FP64, table and -DUSE_CHEBY builds), on
small seeded inputs and records energies, stresses, per-atom values of the
first ids, layout checksums and short trajectories.  The fixtures pin the
CPU oracle (tests/test_oracle.py) on machines where the reference sources
are not available.

Usage: python tests/golden/make_golden.py   (needs oracle/_ref built)
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import ctypes as C  # noqa: E402

from comd_gb300.abi import by_id, occupied_mask, slot_views  # noqa: E402
from oracle import ref_lib  # noqa: E402

POTDIR = os.path.join(ROOT, "comd_gb300", "pots").encode()
EV = 1.0 / 27.211386245988
NIDS = 12


def layout_hash(s):
    v = slot_views(s)
    m = occupied_mask(s)
    h = hashlib.sha256()
    h.update(v["natoms"].astype(np.int32).tobytes())
    h.update(v["id"][m].astype(np.int32).tobytes())
    return h.hexdigest()


def snapshot(s):
    f = by_id(s, "f")
    out = {
        "e": s.contents.e,
        "stress": s.contents.stress,
        "ntot": s.contents.ntot,
        "f_first": f[:NIDS].tolist(),
        "f_abs_sum": float(np.abs(f[:, :3]).sum()),
        "e_atom_sum": float(f[:, 3].sum()),
        "rho_first": by_id(s, "rho")[:NIDS].tolist(),
        "fi_first": by_id(s, "fi")[:NIDS].tolist(),
        "r_first": by_id(s, "r")[:NIDS].tolist(),
        "p_first": by_id(s, "p")[:NIDS].tolist(),
        "layout": layout_hash(s),
    }
    return out


def eam_case(cheby, n, defgrad, bf, seed, kind, amp, temp, steps):
    R = ref_lib(cheby)
    L = R.lib
    pot = L.refh_eam_load(POTDIR, b"cu")
    lat = C.cast(pot, C.POINTER(C.c_double * 8)).contents[7]
    s = L.refh_fcc(n, n, n, lat, defgrad, bf, pot, 1)
    if seed is not None:
        L.refh_seed_apply(s, seed, kind, amp, temp, 63.55)
    L.refh_rebox(s)
    L.refh_force(s)
    out = {"force": snapshot(s)}
    if steps:
        L.refh_ntimesteps(steps, s, 1e-15)
        out["steps"] = steps
        out["after"] = snapshot(s)
    return out


def lj_case(n, sigma, eps, rc, mass, lat, seed, amp, steps):
    R = ref_lib(False)
    L = R.lib
    pot = L.refh_lj_make(sigma, eps, rc, mass)
    s = L.refh_fcc(n, n, n, lat, 1.0, 1.0, pot, 0)
    if seed is not None:
        L.refh_seed_apply(s, seed, 1, amp, 0.0, mass)
    L.refh_rebox(s)
    L.refh_force(s)
    out = {"force": snapshot(s)}
    if steps:
        L.refh_ntimesteps(steps, s, 1e-15)
        out["steps"] = steps
        out["after"] = snapshot(s)
    return out


def clsman_case(cheby, fname, steps):
    """a bundled Ag structure read by the reference's fromFileGzip, reboxed as
    initSimFromCmdLine does, then the force call and `steps` steps"""
    R = ref_lib(cheby)
    L = R.lib
    pot = L.refh_eam_load(POTDIR, b"ag")
    path = os.path.join(ROOT, "comd_gb300", "data", fname).encode()
    s = L.refh_read_clsman(path, 1.0, pot, 1)
    L.refh_rebox(s)
    L.refh_force(s)
    out = {"force": snapshot(s)}
    if steps:
        L.refh_ntimesteps(steps, s, 1e-15)
        out["steps"] = steps
        out["after"] = snapshot(s)
    return out


def file_digests(L, s, tmp):
    """sha256 of the reference's writeClsman bytes, of its gzASCIIWrite text
    (decompressed) and of printIt's output for the state s"""
    import gzip
    out = {}
    L.refh_write_clsman(s, (tmp + ".bin").encode())
    L.refh_gz_ascii_write(s, (tmp + ".txt.gz").encode())
    L.refh_print_it(s, (tmp + ".print").encode())
    b = open(tmp + ".bin", "rb").read()
    t = gzip.open(tmp + ".txt.gz").read()
    pr = open(tmp + ".print", "rb").read()
    out["binary_sha256"] = hashlib.sha256(b).hexdigest()
    out["binary_bytes"] = len(b)
    out["text_sha256"] = hashlib.sha256(t).hexdigest()
    out["text_bytes"] = len(t)
    out["print_sha256"] = hashlib.sha256(pr).hexdigest()
    for ext in (".bin", ".txt.gz", ".print"):
        os.remove(tmp + ext)
    return out


def writer_cases(tmpdir):
    """clsman output of (1) the Ag 8k file as read and reboxed, (2) a seeded
    Cu lattice (displacements and momenta from the shared seed routine) with
    its forces computed, under a set comment"""
    L = ref_lib(False).lib
    pot = L.refh_eam_load(POTDIR, b"ag")
    s = L.refh_read_clsman(os.path.join(ROOT, "comd_gb300", "data", "8k.inp.gz").encode(),
                           1.0, pot, 1)
    L.refh_rebox(s)
    w1 = file_digests(L, s, os.path.join(tmpdir, "w1"))
    pot = L.refh_eam_load(POTDIR, b"cu")
    lat = C.cast(pot, C.POINTER(C.c_double * 8)).contents[7]
    s = L.refh_fcc(6, 6, 6, lat, 1.0, 1.0, pot, 1)
    L.refh_seed_apply(s, 21, 2, 0.05, 600.0, 63.55)
    L.refh_rebox(s)
    L.refh_force(s)
    L.refh_set_comment(s, b"seeded Cu lattice 6x6x6\n")
    w2 = file_digests(L, s, os.path.join(tmpdir, "w2"))
    return {"ag8k_read": w1, "cu6_seeded_forced": w2}


TIM_BOUNDS = (327.42399999999997817, 354.44687726089500757, 3007.58148577889733133)


def tim_file(path, n=400, seed=31):
    """n FileAtom records (x, y, z, bond order, centrosymmetry as float32),
    positions uniform in the reference's fixed bounds"""
    rng = np.random.default_rng(seed)
    rec = np.zeros((n, 5), dtype=np.float32)
    rec[:, :3] = rng.uniform(0.0, 1.0, (n, 3)) * np.array(TIM_BOUNDS)
    rec[:, 3:] = rng.uniform(0.0, 1.0, (n, 2))
    rec.tofile(path)


def tim_case(tmpdir):
    """fromFileTim (read.c:248-315) on a seeded FileAtom file; an LJ potential
    with a 50 A cutoff keeps the fixed bounds' grid small (6 x 7 x 60 boxes)"""
    L = ref_lib(False).lib
    pot = L.refh_lj_make(20.0, 0.01, 50.0, 63.55)
    path = os.path.join(tmpdir, "atoms.tim")
    tim_file(path)
    s = L.refh_read_tim(path.encode(), 1.0, pot)
    v = s.contents
    out = {"ntot": v.ntot, "nbx": list(v.nbx), "layout": layout_hash(s),
           "r_sum": float(np.abs(by_id(s, "r")).sum()), "itype": int(by_id(s, "iType")[0]),
           "mass": float(by_id(s, "mass")[0])}
    os.remove(path)
    return out


def generate():
    """every fixture, computed by the reference (oracle/_ref must be built)"""
    fx = {"generator": "tests/golden/make_golden.py (reference src-flat via oracle/_ref)"}
    # known answers (perfect lattices, as the reference's own runs)
    fx["cu10_table_perfect"] = eam_case(False, 10, 1.0, 1.0, None, 0, 0, 0, 0)
    fx["cu10_cheby_perfect"] = eam_case(True, 10, 1.0, 1.0, None, 0, 0, 0, 0)
    fx["lj20_default_perfect"] = lj_case(20, 1.53, 0.0085, 3 * 1.53, 1.0,
                                         1.122462048 * 3 * 1.53, None, 0, 0)
    # seeded cases with short trajectories
    fx["cu6_table_600K"] = eam_case(False, 6, 1.0, 1.0, 1, 2, 0.05, 600.0, 10)
    fx["cu6_cheby_600K"] = eam_case(True, 6, 1.0, 1.0, 1, 2, 0.05, 600.0, 10)
    fx["cu13_cheby_stretch_bf15"] = eam_case(True, 13, 1.05, 1.5, 3, 2, 0.05, 300.0, 5)
    fx["cu3_table_small_grid"] = eam_case(False, 3, 1.0, 1.0, 4, 2, 0.05, 600.0, 3)
    fx["lj8_default_run_params"] = lj_case(8, 2.315, 0.167 * EV, 2.5 * 2.315, 63.55, 3.615, 5,
                                        0.01 * 2.315, 10)
    # the bundled Ag structures (clsman files)
    fx["ag8k_table_file"] = clsman_case(False, "8k.inp.gz", 10)
    fx["ag8k_cheby_file"] = clsman_case(True, "8k.inp.gz", 10)
    fx["ag262k_table_file"] = clsman_case(False, "262k.inp.gz", 0)
    fx["ag262k_cheby_file"] = clsman_case(True, "262k.inp.gz", 0)
    import tempfile
    with tempfile.TemporaryDirectory() as td:
        fx["clsman_writers"] = writer_cases(td)
        fx["tim_reader"] = tim_case(td)
    return fx


def main():
    if ref_lib(False) is None or ref_lib(True) is None:
        sys.exit("oracle/_ref is not built (run make -C oracle with the reference sources)")
    fx = generate()
    with open(os.path.join(HERE, "reference_fixtures.json"), "w") as f:
        json.dump(fx, f, indent=1)
    print("wrote", os.path.join(HERE, "reference_fixtures.json"))


if __name__ == "__main__":
    main()
