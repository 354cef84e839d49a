"""Centrosymmetry parameter (comdgb_sim_centrosymmetry) against the
reference visualiser's computeCentrosymmetry (src-viz/AtomVisualize.c:
399-672).  The visualiser itself cannot be built here (VTK and OpenGL), but
that one routine is arithmetic on the slot arrays: oracle/Makefile compiles
its text inside a shim without graphics (oracle/_ref/libcomdref_centro*.so)
and tests/golden/make_centro_golden.py records its per-atom values for
fixed inputs in tests/golden/centro_reference.json.  The chain:
  * the oracle's restatement (oracle/centro_oracle.c) equals the reference
    routine bit for bit, live where the shim is built and against the
    fixtures everywhere;
  * the GPU values equal the fixtures and the oracle bit for bit.
Known answers of the physics check the restatement as well: ~0 on a perfect
lattice (the periodic offsets the visualiser rounds to float leave ~1e-12),
and for the 12 neighbours of a vacancy the least pairing of its 11 remaining
nearest neighbours and one second-shell atom at distance a, which is a^2/2,
a^2 or 3a^2/2 depending on which second-shell atom is among the 12."""
import json
import os
import sys

import numpy as np
import pytest

import comd_gb300 as cg
from comd_gb300.abi import occupied_mask, slot_views
from helpers import Case

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
from make_centro_golden import by_id, centro_case, digest, layout_digest  # noqa: E402

FIXTURES = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                        "centro_reference.json")

LAT = 3.615


def perfect(n=6, bf=1.0):
    pot = cg.eam_potential("cu")
    return cg.fcc(n, n, n, pot.ptr.contents.lat, 1.0, bf, pot), pot


def remove_atom(s, atom_id):
    """take atom `atom_id` out of its box (the box's last atom takes its
    slot, as the reference's moveAtom does); returns its world position"""
    v = slot_views(s)
    occ = occupied_mask(s)
    slot = int(np.nonzero((v["id"] == atom_id) & occ)[0][0])
    b = slot // 64
    pos = v["dcenter"][b] + v["r"][slot]
    last = b * 64 + v["natoms"][b] - 1
    for f in ("id", "iType", "mass", "r", "p"):
        v[f][slot] = v[f][last]
    v["natoms"][b] -= 1
    s.contents.ntot -= 1
    return pos


def world(s):
    v = slot_views(s)
    return np.repeat(v["dcenter"], 64, axis=0) + v["r"]


# ---------------------------------------------------------------- CPU ----

def test_oracle_perfect_lattice_is_centrosymmetric(oracle):
    s, _pot = perfect()
    try:
        c, lo, hi = oracle.centro(s)
        m = occupied_mask(s)
        assert np.all(c[m] < 1e-10)
        assert lo == c[m].min() and hi == c[m].max()
        ca, _, _ = oracle.centro(s, approx=True)
        assert np.all(ca[m] < 1e-10)
    finally:
        cg.free_host(s)


def test_oracle_vacancy_neighbours(oracle):
    s, _pot = perfect()
    try:
        hole = remove_atom(s, 100)
        c, _, _ = oracle.centro(s)
        m = occupied_mask(s)
        b = np.array(list(s.contents.bounds))
        d = world(s) - hole
        d -= b * np.round(d / b)
        dist = np.sqrt((d ** 2).sum(axis=1))
        nn = m & (np.abs(dist - LAT / np.sqrt(2)) < 1e-6)
        assert nn.sum() == 12
        allowed = np.array([0.5, 1.0, 1.5]) * LAT ** 2
        for x in c[nn]:
            assert np.min(np.abs(allowed - x)) < 1e-4, x
        far = m & (dist > 2.0 * LAT)
        assert np.all(c[far] < 1e-10)
    finally:
        cg.free_host(s)


def test_oracle_greedy_bounds_the_optimum(oracle):
    """the greedy pairing is a pairing, so never below the least one"""
    c = Case(oracle, cg.POT_EAM_TABLE, n=(6, 6, 6), amp=0.05, temp=600.0)
    try:
        ce, _, _ = oracle.centro(c.s)
        ca, _, _ = oracle.centro(c.s, approx=True)
        m = occupied_mask(c.s)
        assert np.all(ca[m] >= ce[m] * (1 - 1e-5))
        assert ce[m].max() > 0.01
    finally:
        c.close()


def fixture_cases():
    with open(FIXTURES) as f:
        return json.load(f)["cases"]


def check_against_fixture(name, fx, s, compute):
    """compute(s, approx) -> (per-slot values, min, max), checked against the
    reference's recorded values; the range as the routine keeps it (floats,
    maxCentro clamped to 100)"""
    assert layout_digest(s) == fx["input"], f"{name}: input differs from the fixture's"
    for key, approx in (("exact", False), ("approx", True)):
        c, lo, hi = compute(s, approx)
        vals = by_id(s, c)
        want = fx[key]
        assert vals[:len(want["first"])].tolist() == want["first"], (name, key)
        assert digest(vals) == want["sha256"], (name, key)
        assert float(np.float32(lo)) == want["min_centro"], (name, key)
        assert min(float(np.float32(hi)), 100.0) == want["max_centro"], (name, key)


@pytest.mark.parametrize("name", sorted(fixture_cases()))
def test_oracle_centro_matches_reference_fixtures(oracle, name):
    fx = fixture_cases()[name]
    s, _pot = centro_case(fx["spec"])
    try:
        assert s.contents.ntot == fx["ntot"] and list(s.contents.nbx) == fx["nbx"]
        check_against_fixture(name, fx, s, lambda t, a: oracle.centro(t, a))
    finally:
        cg.free_host(s)


@pytest.mark.parametrize("approx", [False, True])
def test_oracle_centro_matches_reference_live(oracle, approx):
    """vacancies, Gaussian-seeded lattices, a 2-box grid and box factor 1.2
    against the reference routine itself, where its shim is built"""
    from oracle import ref_centro
    ref = ref_centro(approx)
    if ref is None:
        pytest.skip("oracle/_ref holds no centrosymmetry build (no reference sources)")
    sims, keep = cases(oracle)
    try:
        for name, s in sims:
            co, lo, hi = oracle.centro(s, approx)
            cr, rlo, rhi = ref.centro(s)
            m = occupied_mask(s)
            assert np.array_equal(co[m].view(np.uint64), cr[m].view(np.uint64)), name
            assert float(np.float32(lo)) == rlo and min(float(np.float32(hi)), 100.0) == rhi, name
    finally:
        release(sims, keep)


# ---------------------------------------------------------------- GPU ----

def gpu_centro(s, approx=False):
    d = cg.DeviceSim(s, cg.opts(cg.POT_EAM_TABLE, cg.PREC_FP64))
    try:
        return d.centrosymmetry(0, approx)
    finally:
        d.close()


def cases(oracle):
    """[(name, host simulation)] for the comparisons, and the Case objects
    that own some of them"""
    out = []
    s, p1 = perfect()
    out.append(("perfect", s))
    s, p2 = perfect()
    remove_atom(s, 100)
    remove_atom(s, 101)
    out.append(("vacancies", s))
    c = Case(oracle, cg.POT_EAM_TABLE, n=(6, 6, 6), amp=0.05, temp=600.0)
    out.append(("thermal", c.s))
    c2 = Case(oracle, cg.POT_EAM_TABLE, n=(4, 4, 4), amp=0.05, temp=600.0)  # 2 boxes per axis
    out.append(("small grid", c2.s))
    c3 = Case(oracle, cg.POT_EAM_TABLE, n=(6, 7, 6), bf=1.2, amp=0.08, temp=1200.0)
    out.append(("bf 1.2", c3.s))
    ag_pot = cg.eam_potential("ag")
    ag = cg.read_clsman(os.path.join(cg.DATA_DIR, "8k.inp.gz"), ag_pot, 1.0, -1)
    out.append(("Ag 8k", ag))
    return out, [c, c2, c3, ag_pot, p1, p2]


def release(sims, keep):
    for name, s in sims:
        if name in ("perfect", "vacancies", "Ag 8k"):
            cg.free_host(s)
    for c in keep:
        if isinstance(c, Case):
            c.close()


@pytest.mark.gpu
@pytest.mark.parametrize("approx", [False, True])
def test_gpu_centro_matches_oracle_bitwise(oracle, approx):
    sims, keep = cases(oracle)
    try:
        for name, s in sims:
            co, lo, hi = oracle.centro(s, approx)
            cgpu, glo, ghi = gpu_centro(s, approx)
            m = occupied_mask(s)
            assert np.array_equal(cgpu[m], co[m]), name
            assert np.all(cgpu[~m] == 0), name
            assert (glo, ghi) == (lo, hi), name
    finally:
        release(sims, keep)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(fixture_cases()))
def test_gpu_centro_matches_reference_fixtures(name):
    fx = fixture_cases()[name]
    s, _pot = centro_case(fx["spec"])
    try:
        check_against_fixture(name, fx, s, gpu_centro)
    finally:
        cg.free_host(s)


@pytest.mark.gpu
def test_gpu_batch_centro_equals_single(oracle):
    from test_batch import make_replicas
    pot = cg.eam_potential("cu")
    bs = make_replicas(pot)
    try:
        b = cg.Batch(bs, cg.opts(cg.POT_EAM_TABLE, cg.PREC_FP64))
        try:
            got = [b.centrosymmetry(r) for r in range(b.n)]
        finally:
            b.close()
        for r, s in enumerate(bs):
            co, lo, hi = oracle.centro(s)
            m = occupied_mask(s)
            assert np.array_equal(got[r][0][m], co[m]), r
            assert (got[r][1], got[r][2]) == (lo, hi), r
    finally:
        for s in bs:
            cg.free_host(s)
