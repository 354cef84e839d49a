"""CPU tests pinning the oracle (oracle/comd_oracle.c) to the reference.

1. Known answers of the reference's own runs (perfect lattices).
2. The committed fixtures generated by the reference itself
   (tests/golden/make_golden.py, compiled from the reference sources).
3. Where the reference sources are present (oracle/_ref built), a
   byte-for-byte comparison of every slot array after force, reBoxAll and
   several timesteps.
"""
import numpy as np
import pytest

from comd_gb300.abi import slot_views
from helpers import FIX, match, snapshot
from oracle import KIND_EAM_CHEBY, KIND_EAM_TABLE, KIND_LJ, ref_lib

EV = 1.0 / 27.211386245988


def eam_run(oracle, pots_dir, cheby, n, defgrad, bf, seed, kind, amp, temp, steps):
    pot = oracle.eam(pots_dir, "cu")
    s = oracle.fcc(n, n, n, pot.contents.lat, defgrad, bf, pot)
    s.contents.ch_pot = oracle.cheby(pot, 32)
    if seed is not None:
        oracle.seed(s, seed, kind, amp, temp, 63.55)
    assert oracle.rebox(s) == 0
    k = KIND_EAM_CHEBY if cheby else KIND_EAM_TABLE
    assert oracle.force(s, k) == 0
    snap = snapshot(s)
    after = None
    if steps:
        assert oracle.steps(s, steps, 1e-15, k) == 0
        after = snapshot(s)
    oracle.free(s)
    return snap, after


def lj_run(oracle, n, sigma, eps, rc, mass, lat, seed, amp, steps):
    pot = oracle.lj(sigma, eps, rc, mass)
    s = oracle.fcc(n, n, n, lat, 1.0, 1.0, pot)
    if seed is not None:
        oracle.seed(s, seed, 1, amp, 0.0, mass)
    assert oracle.rebox(s) == 0
    assert oracle.force(s, KIND_LJ) == 0
    snap = snapshot(s)
    after = None
    if steps:
        assert oracle.steps(s, steps, 1e-15, KIND_LJ) == 0
        after = snapshot(s)
    oracle.free(s)
    return snap, after


def test_known_answer_cu_table_10(oracle, pots_dir):
    """comd -e -p cu -x 10 -y 10 -z 10 (reference run): E = -520.39690803365010652 Ha."""
    snap, _ = eam_run(oracle, pots_dir, False, 10, 1.0, 1.0, None, 0, 0, 0, 0)
    assert snap["e"] == pytest.approx(-520.39690803365010652, rel=1e-15)
    assert snap["stress"] == pytest.approx(-0.0307682, rel=1e-5)


def test_known_answer_lj_default_20(oracle):
    """comd (LJ defaults, 20^3): E = -35.622392760664631 Ha."""
    snap, _ = lj_run(oracle, 20, 1.53, 0.0085, 3 * 1.53, 1.0, 1.122462048 * 3 * 1.53, None, 0,
                     0)
    assert snap["e"] == pytest.approx(-35.622392760664631, rel=1e-14)


def test_known_answer_cu_40(oracle, pots_dir):
    """comd -e -p cu 40^3: table -33305.402116232784, Chebyshev -33304.291406184107."""
    snap, _ = eam_run(oracle, pots_dir, False, 40, 1.0, 1.0, None, 0, 0, 0, 0)
    assert snap["e"] == pytest.approx(-33305.402116232784, rel=1e-14)
    snap, _ = eam_run(oracle, pots_dir, True, 40, 1.0, 1.0, None, 0, 0, 0, 0)
    assert snap["e"] == pytest.approx(-33304.291406184107, rel=1e-13)


EAM_CASES = {
    "cu10_table_perfect": (False, 10, 1.0, 1.0, None, 0, 0, 0, 0),
    "cu10_cheby_perfect": (True, 10, 1.0, 1.0, None, 0, 0, 0, 0),
    "cu6_table_600K": (False, 6, 1.0, 1.0, 1, 2, 0.05, 600.0, 10),
    "cu6_cheby_600K": (True, 6, 1.0, 1.0, 1, 2, 0.05, 600.0, 10),
    "cu13_cheby_stretch_bf15": (True, 13, 1.05, 1.5, 3, 2, 0.05, 300.0, 5),
    "cu3_table_small_grid": (False, 3, 1.0, 1.0, 4, 2, 0.05, 600.0, 3),
}


@pytest.mark.parametrize("name", sorted(EAM_CASES))
def test_oracle_matches_reference_fixture_eam(oracle, pots_dir, name):
    snap, after = eam_run(oracle, pots_dir, *EAM_CASES[name])
    match(snap, FIX[name]["force"])
    if after is not None:
        match(after, FIX[name]["after"], rtol=1e-11)


def test_oracle_matches_reference_fixture_lj(oracle):
    snap, after = lj_run(oracle, 8, 2.315, 0.167 * EV, 2.5 * 2.315, 63.55, 3.615, 5,
                         0.01 * 2.315, 10)
    match(snap, FIX["lj8_default_run_params"]["force"])
    match(after, FIX["lj8_default_run_params"]["after"], rtol=1e-11)


@pytest.mark.parametrize("cheby", [False, True])
def test_oracle_bitexact_vs_compiled_reference(oracle, pots_dir, cheby):
    R = ref_lib(cheby)
    if R is None:
        pytest.skip("reference sources not available here (oracle/_ref not built)")
    L = R.lib
    k = KIND_EAM_CHEBY if cheby else KIND_EAM_TABLE
    rp = L.refh_eam_load(pots_dir.encode(), b"cu")
    pot = oracle.eam(pots_dir, "cu")
    for n, dg, bf in ((6, 1.0, 1.0), (13, 1.05, 1.5), (3, 1.0, 1.0)):
        rs = L.refh_fcc(n, n, n, pot.contents.lat, dg, bf, rp, 1)
        s = oracle.fcc(n, n, n, pot.contents.lat, dg, bf, pot)
        s.contents.ch_pot = oracle.cheby(pot, 32)
        L.refh_seed_apply(rs, 7, 2, 0.08, 900.0, 63.55)
        oracle.seed(s, 7, 2, 0.08, 900.0, 63.55)
        L.refh_rebox(rs)
        assert oracle.rebox(s) == 0
        L.refh_force(rs)
        assert oracle.force(s, k) == 0
        va, vb = slot_views(s), slot_views(rs)
        for f in va:
            assert np.array_equal(va[f], vb[f]), f
        assert s.contents.e == rs.contents.e and s.contents.stress == rs.contents.stress
        L.refh_ntimesteps(8, rs, 1e-15)
        assert oracle.steps(s, 8, 1e-15, k) == 0
        for f in va:
            assert np.array_equal(va[f], vb[f]), f
        assert s.contents.e == rs.contents.e
        oracle.free(s)


def test_committed_fixtures_regenerate_from_the_reference():
    """tests/golden/reference_fixtures.json is exactly what the reference
    computes today: make_golden.generate() on the reference compiled from its
    sources reproduces every committed value (skipped where the reference
    sources are absent)."""
    import json
    import os
    import sys
    if ref_lib(False) is None or ref_lib(True) is None:
        pytest.skip("reference sources not present (oracle/_ref not built)")
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    sys.path.insert(0, here)
    import make_golden
    fresh = json.loads(json.dumps(make_golden.generate()))
    with open(os.path.join(here, "reference_fixtures.json")) as f:
        committed = json.load(f)
    assert fresh.keys() == committed.keys()
    for k in committed:
        assert fresh[k] == committed[k], k
