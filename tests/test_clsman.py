"""clsman input (fromFileGzip, read.c:155-241) on the bundled Ag structures.

Known answers from runs of the reference on data/8k.inp.gz with the Ag
potential, box factor 1 (`comd_dbl -e -p ag -f data/8k.inp.gz` and the
Chebyshev build): E0 (after the first force call), E10 (after nTimeSteps(10),
dt = 1 fs, table) and E200 (after 20 x nTimeSteps(10), Chebyshev)."""
import gzip
import os

import numpy as np
import pytest

import comd_gb300 as cg
from comd_gb300.abi import by_id
from helpers import FIX, match, slots_equal, snapshot
from oracle import KIND_EAM_CHEBY, KIND_EAM_TABLE

E0_TABLE = -852.31072722864178
E10_TABLE = -852.67331452789108
E0_CHEBY = -852.27037691173302
E200_CHEBY = -854.77081758005625
E0_TWO_ATOMS = -0.007229952672898890681
GZ = os.path.join(cg.DATA_DIR, "8k.inp.gz")


# fixture name -> (file, Chebyshev?, steps after the force call)
FILE_CASES = {"ag8k_table_file": ("8k.inp.gz", False, 10),
              "ag8k_cheby_file": ("8k.inp.gz", True, 10),
              "ag262k_table_file": ("262k.inp.gz", False, 0),
              "ag262k_cheby_file": ("262k.inp.gz", True, 0)}


@pytest.fixture(scope="module")
def text_dir(tmp_path_factory):
    """the bundled files decompressed (the oracle reads text)"""
    d = tmp_path_factory.mktemp("clsman")
    for f in ("8k.inp.gz", "262k.inp.gz", "2.inp.gz"):
        (d / f[:-3]).write_bytes(gzip.open(os.path.join(cg.DATA_DIR, f)).read())
    return d


@pytest.fixture(scope="module")
def text_file(text_dir):
    return str(text_dir / "8k.inp")


def zlib_built():
    pot = cg.eam_potential("ag")
    try:
        s = cg.read_clsman(GZ, pot, 1.0, -1)
    except cg.ComdgbError as e:
        if e.code == -34:
            return False
        raise
    cg.free_host(s)
    return True


def host_read(text_file, pot):
    return cg.read_clsman(GZ if zlib_built() else text_file, pot, 1.0, -1)


def test_oracle_clsman_known_answers(oracle, pots_dir, text_file):
    opot = oracle.eam(pots_dir, "ag")
    for kind, e0 in [(KIND_EAM_TABLE, E0_TABLE), (KIND_EAM_CHEBY, E0_CHEBY)]:
        so = oracle.read_clsman(text_file, opot, 1.0)
        try:
            assert so.contents.ntot == 8192
            if kind == KIND_EAM_CHEBY:
                so.contents.ch_pot = oracle.cheby(opot, 32)
            assert oracle.rebox(so) == 0
            assert oracle.force(so, kind) == 0
            assert so.contents.e == pytest.approx(e0, rel=1e-15, abs=0)
        finally:
            oracle.free(so)


def test_oracle_two_atom_file(oracle, pots_dir, text_dir):
    so = oracle.read_clsman(str(text_dir / "2.inp"), oracle.eam(pots_dir, "ag"), 1.0)
    try:
        assert so.contents.ntot == 2
        assert oracle.rebox(so) == 0
        assert oracle.force(so, KIND_EAM_TABLE) == 0
        assert so.contents.e == pytest.approx(E0_TWO_ATOMS, rel=1e-14, abs=0)
    finally:
        oracle.free(so)


@pytest.mark.parametrize("name", sorted(FILE_CASES))
def test_oracle_matches_reference_fixture_files(oracle, pots_dir, text_dir, name):
    """the oracle on the bundled structures against the reference's own runs
    (tests/golden/make_golden.py): layout, energy, stress, forces, and the
    state after 10 steps for the 8k file"""
    fname, cheby, steps = FILE_CASES[name]
    opot = oracle.eam(pots_dir, "ag")
    so = oracle.read_clsman(str(text_dir / fname[:-3]), opot, 1.0)
    kind = KIND_EAM_CHEBY if cheby else KIND_EAM_TABLE
    try:
        if cheby:
            so.contents.ch_pot = oracle.cheby(opot, 32)
        assert oracle.rebox(so) == 0
        assert oracle.force(so, kind) == 0
        match(snapshot(so), FIX[name]["force"])
        if steps:
            assert oracle.steps(so, steps, 1e-15, kind) == 0
            match(snapshot(so), FIX[name]["after"], rtol=1e-11)
    finally:
        oracle.free(so)


def test_host_reader_matches_oracle_and_reference(oracle, pots_dir, text_file):
    pot = cg.eam_potential("ag")
    sh = host_read(text_file, pot)
    so = oracle.read_clsman(text_file, oracle.eam(pots_dir, "ag"), 1.0)
    try:
        assert sh.contents.ntot == 8192
        assert list(sh.contents.nbx) == [11, 11, 5]
        assert slots_equal(sh, so, ("id", "iType", "mass", "r", "p"))
        try:
            from oracle import ref_lib
            ref = ref_lib(False)
        except (FileNotFoundError, OSError):
            return  # the reference sources are not on this machine
        ep = ref.lib.refh_eam_load(pots_dir.encode(), b"ag")
        sr = ref.lib.refh_read_clsman(GZ.encode(), 1.0, ep, 0)
        assert slots_equal(sh, sr, ("id", "iType", "mass", "r", "p"))
    finally:
        cg.free_host(sh)
        oracle.free(so)


def test_host_reader_262k_matches_oracle(oracle, pots_dir, text_dir):
    """the 262,144-atom file, whose atom lines the library parses on 16
    threads: the same slots as the oracle's serial reader"""
    pot = cg.eam_potential("ag")
    path = str(text_dir / "262k.inp")
    sh = cg.read_clsman(path, pot, 1.0, -1)
    so = oracle.read_clsman(path, oracle.eam(pots_dir, "ag"), 1.0)
    try:
        assert sh.contents.ntot == 262144
        assert slots_equal(sh, so, ("id", "iType", "mass", "r", "p"))
    finally:
        cg.free_host(sh)
        oracle.free(so)


def test_host_reader_reports_a_bad_atom_line(oracle, tmp_path, text_dir):
    """a malformed atom line in the middle of a large file is an I/O error
    (-33), as a short file is, whichever thread parses it"""
    pot = cg.eam_potential("ag")
    lines = (text_dir / "262k.inp").read_text().split("\n")
    lines[3 + 200000] = "1.0 2.0 x"
    bad = tmp_path / "bad.inp"
    bad.write_text("\n".join(lines))
    with pytest.raises(cg.ComdgbError) as ei:
        cg.read_clsman(str(bad), pot, 1.0, -1)
    assert ei.value.code == -33  # COMDGB_ERR_IO
    short = tmp_path / "short.inp"
    short.write_text("\n".join(lines[:3 + 1000]))
    with pytest.raises(cg.ComdgbError) as ei:
        cg.read_clsman(str(short), pot, 1.0, -1)
    assert ei.value.code == -33


@pytest.mark.gpu
def test_gpu_binning_of_clsman_file_matches_host(text_file):
    pot = cg.eam_potential("ag")
    src = GZ if zlib_built() else text_file
    sd = cg.read_clsman(src, pot, 1.0, 0)
    sh = cg.read_clsman(src, pot, 1.0, -1)
    try:
        assert slots_equal(sd, sh, ("id", "iType", "mass", "r", "p"))
    finally:
        cg.free_host(sd)
        cg.free_host(sh)


@pytest.mark.gpu
@pytest.mark.parametrize("potential", [cg.POT_EAM_TABLE, cg.POT_EAM_CHEBY])
def test_gpu_clsman_known_answers(text_file, potential):
    pot = cg.eam_potential("ag")
    s = host_read(text_file, pot)
    try:
        assert cg.load().comdgb_rebox_host(s, 1, 0) == 0
        d = cg.DeviceSim(s, cg.opts(potential, cg.PREC_FP64))
        try:
            e0 = d.force()[0]
            if potential == cg.POT_EAM_TABLE:
                assert e0 == pytest.approx(E0_TABLE, rel=1e-13, abs=0)
                assert d.steps(10)[0] == pytest.approx(E10_TABLE, rel=1e-10, abs=0)
            else:
                assert e0 == pytest.approx(E0_CHEBY, rel=1e-12, abs=0)
                for _ in range(20):
                    e = d.steps(10)[0]
                assert e == pytest.approx(E200_CHEBY, rel=1e-8, abs=0)
        finally:
            d.close()
    finally:
        cg.free_host(s)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(FILE_CASES))
def test_gpu_matches_reference_fixture_files(text_dir, name):
    """device-binned read, FP64 force (and 10 steps on the 8k file) against
    the reference's own runs on the same files"""
    fname, cheby, steps = FILE_CASES[name]
    pot = cg.eam_potential("ag")
    src = os.path.join(cg.DATA_DIR, fname) if zlib_built() else str(text_dir / fname[:-3])
    s = cg.read_clsman(src, pot, 1.0, 0)
    try:
        assert cg.load().comdgb_rebox_host(s, 1, 0) == 0
        d = cg.DeviceSim(s, cg.opts(cg.POT_EAM_CHEBY if cheby else cg.POT_EAM_TABLE,
                                    cg.PREC_FP64, True, per_step_lists=True))
        try:
            d.force()
            d.download(s)
            match(snapshot(s), FIX[name]["force"])
            if steps:
                d.steps(steps, 1e-15)
                d.download(s)
                match(snapshot(s), FIX[name]["after"], rtol=1e-10, vrtol=1e-10)
        finally:
            d.close()
    finally:
        cg.free_host(s)


@pytest.mark.gpu
def test_gpu_mixed_forces_on_clsman_structure(text_file):
    """mixed precision on the real Ag structure: force error vs FP64 < 1e-5"""
    pot = cg.eam_potential("ag")
    s64, s32 = host_read(text_file, pot), host_read(text_file, pot)
    try:
        for s in (s64, s32):
            assert cg.load().comdgb_rebox_host(s, 1, 0) == 0
        for s, prec in ((s64, cg.PREC_FP64), (s32, cg.PREC_MIXED)):
            d = cg.DeviceSim(s, cg.opts(cg.POT_EAM_CHEBY, prec))
            try:
                d.force()
                d.download(s)
            finally:
                d.close()
        f64 = by_id(s64, "f")[:, :3]
        f32 = by_id(s32, "f")[:, :3]
        err = np.sqrt(((f32 - f64) ** 2).sum() / (f64 ** 2).sum())
        assert err < 1e-5
    finally:
        cg.free_host(s64)
        cg.free_host(s32)


# ------------------------------------------------ FileAtom reader ----

def tim_setup(tmp_path):
    """the seeded FileAtom file of the reference fixture and its LJ potential
    (50 A cutoff: 6 x 7 x 60 boxes over the reference's fixed bounds)"""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    from make_golden import tim_file
    path = str(tmp_path / "atoms.tim")
    tim_file(path)
    return path, cg.lj_potential(20.0, 0.01, 50.0, 63.55)


def check_tim(s):
    from helpers import layout_hash
    ref = FIX["tim_reader"]
    v = s.contents
    assert v.ntot == ref["ntot"] and list(v.nbx) == ref["nbx"]
    assert layout_hash(s) == ref["layout"]
    assert float(np.abs(by_id(s, "r")).sum()) == ref["r_sum"]
    assert np.all(by_id(s, "iType") == 1) and np.all(by_id(s, "mass") == ref["mass"])
    assert np.all(by_id(s, "p") == 0)


def test_tim_reader_host_matches_reference(tmp_path):
    path, pot = tim_setup(tmp_path)
    s = cg.read_tim(path, pot, 1.0, None, -1)
    try:
        check_tim(s)
        try:
            from oracle import ref_lib
            ref = ref_lib(False)
        except (FileNotFoundError, OSError):
            return  # the reference sources are not on this machine
        rp = ref.lib.refh_lj_make(20.0, 0.01, 50.0, 63.55)
        sr = ref.lib.refh_read_tim(path.encode(), 1.0, rp)
        assert slots_equal(s, sr, ("id", "iType", "mass", "r", "p"))
    finally:
        cg.free_host(s)


def test_tim_reader_bounds_override(tmp_path):
    path, pot = tim_setup(tmp_path)
    s = cg.read_tim(path, pot, 1.0, (400.0, 400.0, 3100.0), -1)
    try:
        assert list(s.contents.bounds) == [400.0, 400.0, 3100.0]
        assert s.contents.ntot == 400
    finally:
        cg.free_host(s)


@pytest.mark.gpu
def test_tim_reader_device_binning(tmp_path):
    path, pot = tim_setup(tmp_path)
    sd = cg.read_tim(path, pot, 1.0, None, 0)
    try:
        check_tim(sd)
    finally:
        cg.free_host(sd)
