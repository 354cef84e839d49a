"""GPU parity: the library's CUDA path against the CPU oracle on the same
seeded inputs (all calls go through the C ABI of libcomdgb.so).

Tolerances: the FP64 kernels differ from the oracle only in the order of the
per-atom sums, so forces agree to 1e-11 of the largest component and energy
to 1e-12 relative.  Integer work (box occupancy, slot order, ids) and the
FP64 integrator are bit-exact.  Mixed precision must stay within the
1e-5 relative RMS force error of the specification.
"""
import ctypes as C

import numpy as np
import pytest

import comd_gb300 as cg
from comd_gb300.abi import by_id, occupied_mask, slot_views
from helpers import Case, compare_forces, layout_equal, rel_rms, slots_equal, world_by_id

pytestmark = pytest.mark.gpu

FP64_F_TOL = 1e-11
FP64_E_TOL = 1e-12
MIXED_F_RMS_TOL = 1e-5


def _force_case(oracle, potential, precision, **kw):
    c = Case(oracle, potential, **kw)
    try:
        c.oracle_force()
        d = c.device(precision)
        e, stress = d.force()
        d.download(c.s)
        d.close()
        cmp = compare_forces(c.s, c.o)
        eo, so = c.o.contents.e, c.o.contents.stress
        return cmp, (e, stress), (eo, so), c.s.contents.ntot
    finally:
        c.close()


@pytest.mark.parametrize("potential", [cg.POT_EAM_TABLE, cg.POT_EAM_CHEBY])
def test_eam_force_fp64(oracle, potential):
    cmp, (e, st), (eo, so), _ = _force_case(oracle, potential, cg.PREC_FP64)
    assert cmp["f_max_rel"] < FP64_F_TOL, cmp
    assert cmp["e_max_rel"] < FP64_F_TOL, cmp
    assert cmp["rho_max_rel"] < FP64_E_TOL, cmp
    assert cmp["fi_max_rel"] < FP64_E_TOL, cmp
    assert abs(e - eo) <= FP64_E_TOL * abs(eo)
    assert abs(st - so) <= 1e-10 * abs(so)


def test_lj_force_fp64(oracle):
    cmp, (e, st), (eo, so), _ = _force_case(oracle, cg.POT_LJ, cg.PREC_FP64, n=(8, 8, 8),
                                            disp=cg.DISP_UNIFORM, amp=0.01 * 2.315, temp=300.0)
    assert cmp["f_max_rel"] < FP64_F_TOL, cmp
    assert cmp["e_max_rel"] < FP64_F_TOL, cmp
    assert abs(e - eo) <= FP64_E_TOL * abs(eo)
    assert abs(st - so) <= 1e-10 * abs(so)


@pytest.mark.parametrize("n", [(3, 3, 3), (2, 2, 2), (2, 5, 4)])
def test_eam_force_small_grids(oracle, n):
    """nbx < 3 (duplicate stencil entries) and a single box, as the reference."""
    cmp, (e, st), (eo, so), _ = _force_case(oracle, cg.POT_EAM_TABLE, cg.PREC_FP64, n=n)
    assert cmp["f_max_rel"] < FP64_F_TOL, cmp
    assert abs(e - eo) <= FP64_E_TOL * abs(eo)


def test_eam_force_nonperiodic(oracle):
    cmp, (e, st), (eo, so), _ = _force_case(oracle, cg.POT_EAM_TABLE, cg.PREC_FP64,
                                            periodic=False)
    assert cmp["f_max_rel"] < FP64_F_TOL, cmp
    assert abs(e - eo) <= FP64_E_TOL * abs(eo)


def test_eam_force_stretched_boxfactor(oracle):
    cmp, (e, st), (eo, so), _ = _force_case(oracle, cg.POT_EAM_CHEBY, cg.PREC_FP64,
                                            n=(13, 13, 13), defgrad=1.05, bf=1.5, temp=300.0,
                                            amp=0.05, disp=cg.DISP_GAUSSIAN)
    assert cmp["f_max_rel"] < FP64_F_TOL, cmp
    assert abs(e - eo) <= FP64_E_TOL * abs(eo)


@pytest.mark.parametrize("potential", [cg.POT_EAM_TABLE, cg.POT_EAM_CHEBY])
def test_eam_force_mixed(oracle, potential):
    cmp, (e, st), (eo, so), ntot = _force_case(oracle, potential, cg.PREC_MIXED,
                                               n=(13, 13, 13), defgrad=1.05, bf=1.5,
                                               temp=300.0, amp=0.05)
    assert cmp["f_rel_rms"] < MIXED_F_RMS_TOL, cmp
    assert abs(e - eo) / ntot < 1e-7, (e, eo)


def test_lj_force_mixed(oracle):
    cmp, (e, st), (eo, so), ntot = _force_case(oracle, cg.POT_LJ, cg.PREC_MIXED, n=(8, 8, 8),
                                               disp=cg.DISP_UNIFORM, amp=0.01 * 2.315)
    assert cmp["f_rel_rms"] < MIXED_F_RMS_TOL, cmp
    assert abs(e - eo) / ntot < 1e-7, (e, eo)


def test_rebox_bitexact(oracle):
    """GPU reBoxAll reproduces occupancy, slot order and every moved field."""
    c = Case(oracle, cg.POT_EAM_TABLE, n=(8, 8, 8), disp=cg.DISP_NONE, amp=0.0)
    try:
        v = slot_views(c.s)
        rng = np.random.default_rng(5)
        v["r"][:] += rng.uniform(-0.9, 0.9, size=v["r"].shape)
        v["f"][:] = rng.normal(size=v["f"].shape)
        v["rho"][:] = rng.normal(size=v["rho"].shape)
        o2 = c.oracle.clone(c.s)
        assert c.oracle.rebox(o2) == 0
        d = c.device()
        d.rebox()
        d.download(c.s)
        d.close()
        assert slots_equal(c.s, o2, ("id", "iType", "mass", "r", "p", "f", "rho", "fi"))
        c.oracle.free(o2)
    finally:
        c.close()


@pytest.mark.parametrize("mass", [63.55, 107.9, 1.0])
def test_integrator_bitexact(oracle, mass):
    """advanceVelocity + advancePositions (+ reBoxAll) equal the oracle bit for bit."""
    c = Case(oracle, cg.POT_EAM_TABLE, n=(8, 8, 8), temp=900.0)
    try:
        c.pot.ptr.contents.mass = mass
        v = slot_views(c.s)
        rng = np.random.default_rng(9)
        v["f"][:] = rng.normal(scale=0.05, size=v["f"].shape)
        v["p"][:] *= 40.0  # large momenta so that atoms cross boxes
        o2 = c.oracle.clone(c.s)
        dt = 1e-15 * cg.lib.BOHR_PER_ATU
        d = c.device()
        d.advance_velocity(dt)
        d.advance_positions(dt / 2.0)
        d.download(c.s)
        d.close()
        c.oracle.lib.orc_advance_velocity(o2, dt)
        c.oracle.lib.orc_advance_positions(o2, dt / 2.0)
        assert c.oracle.rebox(o2) == 0
        assert slots_equal(c.s, o2, ("id", "r", "p", "f"))
        c.oracle.free(o2)
    finally:
        c.close()


def test_rebox_serial_fallback(oracle):
    """Moves of more than one box per axis replay reBoxAll serially, still exact."""
    c = Case(oracle, cg.POT_EAM_TABLE, n=(8, 8, 8), disp=cg.DISP_NONE, amp=0.0)
    try:
        v = slot_views(c.s)
        bs = c.s.contents.boxsize[0]
        nb = c.s.contents.nboxes
        # atoms of box 0 pushed 2.5 boxes up in x: they arrive at box 1 still out of range
        v["r"][0:3, 0] += 2.5 * bs
        v["r"][64 * (nb // 2) + 1, 1] -= 1.7 * c.s.contents.boxsize[1]
        o2 = c.oracle.clone(c.s)
        assert c.oracle.rebox(o2) == 0
        d = c.device()
        d.rebox()
        d.download(c.s)
        d.close()
        assert slots_equal(c.s, o2)
        c.oracle.free(o2)
    finally:
        c.close()


@pytest.mark.parametrize("precision", [cg.PREC_FP64, cg.PREC_MIXED])
def test_persistent_lists_after_serial_rebin(oracle, precision):
    """Persistent lists read neighbours through the id -> slot map the rebin
    keeps.  Moves of more than one box (here 1.7 boxes in x for every fifth
    atom, -1.3 in y for the next) go through the serial replay of reBoxAll,
    which also empties boxes by moving their last atom; the force call after
    it must equal a fresh build's on the same state, and the oracle's."""
    c = Case(oracle, cg.POT_EAM_CHEBY, n=(8, 8, 8), amp=0.05, temp=300.0)
    try:
        v = slot_views(c.s)
        m = occupied_mask(c.s)
        ids = v["id"]
        rmass = c.pot.ptr.contents.mass * cg.lib.AMU_TO_ME
        bs = list(c.s.contents.boxsize)
        dt = 10.0  # internal time units
        sel = m & (ids % 5 == 0)
        v["p"][sel, 0] = 1.7 * bs[0] * rmass / dt
        sel = m & (ids % 5 == 1)
        v["p"][sel, 1] = -1.3 * bs[1] * rmass / dt
        slot_views(c.o)["p"][:] = v["p"]  # the oracle clone has the same layout
        d = cg.DeviceSim(c.s, cg.opts(cg.POT_EAM_CHEBY, precision, True, cheby_from_host=True))
        try:
            assert d.list_info()[0]
            d.force()
            d.advance_positions(dt)
            e1 = d.force()[0]
            d.download(c.s)
        finally:
            d.close()
        f1 = by_id(c.s, "f")[:, :3].copy()
        fresh = cg.DeviceSim(c.s, cg.opts(cg.POT_EAM_CHEBY, precision, True,
                                          cheby_from_host=True))
        try:
            e2 = fresh.force()[0]
            fresh.download(c.s)
        finally:
            fresh.close()
        f2 = by_id(c.s, "f")[:, :3]
        assert abs(e1 - e2) <= 1e-12 * abs(e2), (e1, e2)
        assert np.abs(f1 - f2).max() <= 1e-9 * np.abs(f2).max()
        c.oracle.lib.orc_advance_positions(c.o, dt)
        assert c.oracle.rebox(c.o) == 0
        assert layout_equal(c.s, c.o)
        c.oracle_force()
        eo = c.o.contents.e
        if precision == cg.PREC_FP64:
            assert abs(e1 - eo) <= FP64_E_TOL * abs(eo), (e1, eo)
        else:
            assert abs(e1 - eo) / c.s.contents.ntot < 1e-7, (e1, eo)
    finally:
        c.close()


def test_rebox_overflow_reported(oracle):
    """A box reaching 64 atoms returns the reference's -11 instead of exiting."""
    c = Case(oracle, cg.POT_EAM_TABLE, n=(8, 8, 8), disp=cg.DISP_NONE, amp=0.0)
    try:
        v = slot_views(c.s)
        nbx = list(c.s.contents.nbx)
        bs = list(c.s.contents.boxsize)

        def box(ix, iy, iz):
            return ix + nbx[0] * (iy + nbx[1] * iz)

        # every atom of four face neighbours of box 0 is pushed into box 0
        for b, axis, target in ((box(1, 0, 0), 0, -0.5), (box(0, 1, 0), 1, -0.5),
                                (box(0, 0, 1), 2, -0.5), (box(nbx[0] - 1, 0, 0), 0, 1.5)):
            n = v["natoms"][b]
            v["r"][64 * b:64 * b + n, axis] = target * bs[axis]
        assert v["natoms"][[0, box(1, 0, 0), box(0, 1, 0), box(0, 0, 1),
                            box(nbx[0] - 1, 0, 0)]].sum() >= 64
        o2 = c.oracle.clone(c.s)
        assert c.oracle.rebox(o2) == -11
        d = c.device()
        with pytest.raises(cg.ComdgbError) as ei:
            d.rebox()
        assert ei.value.code == -11
        d.close()
        c.oracle.free(o2)
    finally:
        c.close()


@pytest.mark.parametrize("potential", [cg.POT_EAM_TABLE, cg.POT_EAM_CHEBY, cg.POT_LJ])
def test_steps_fp64(oracle, potential):
    kw = {}
    if potential == cg.POT_LJ:
        kw = dict(n=(8, 8, 8), disp=cg.DISP_UNIFORM, amp=0.01 * 2.315, temp=0.0)
    c = Case(oracle, potential, **kw)
    try:
        nsteps = 10
        d = c.device()
        e, _ = d.steps(nsteps, 1e-15)
        d.download(c.s)
        d.close()
        assert c.oracle.steps(c.o, nsteps, 1e-15, c.kind) == 0
        eo = c.o.contents.e
        assert abs(e - eo) <= 1e-10 * abs(eo), (e, eo)
        assert layout_equal(c.s, c.o)
        rg, ro = by_id(c.s, "r"), by_id(c.o, "r")
        assert np.max(np.abs(rg - ro)) < 1e-9
        pg, po = by_id(c.s, "p"), by_id(c.o, "p")
        assert rel_rms(pg, po) < 1e-8
    finally:
        c.close()


def test_mixed_energy_drift(oracle):
    """Mixed-precision EAM (Chebyshev) conserves H to 1e-4 eV/atom over 1000 steps."""
    c = Case(oracle, cg.POT_EAM_CHEBY, n=(8, 8, 8), temp=600.0, amp=0.05)
    try:
        d = c.device(cg.PREC_MIXED)
        n = c.s.contents.ntot
        e0, _ = d.force()
        h0 = e0 + d.kinetic()
        hs = []
        for _ in range(10):
            e, _ = d.steps(100, 1e-15)
            hs.append(e + d.kinetic())
        d.close()
        drift = max(abs(h - h0) for h in hs) / n
        assert drift < 1e-4 * cg.lib.EV_TO_HA, drift
    finally:
        c.close()


def test_cheb_fit_on_gpu(oracle, pots_dir):
    L = cg.load()
    pot = cg.eam_potential("cu")
    cg_cheb = L.comdgb_cheb_make(pot.ptr, 32, 0)
    assert cg_cheb
    ref = oracle.cheby(oracle.eam(pots_dir, "cu"), 32)
    for name in ("phi", "rho", "f", "dphi", "drho", "df"):
        a = getattr(cg_cheb.contents, name).contents
        b = getattr(ref.contents, name).contents
        va = np.ctypeslib.as_array(a.values, (32,))
        vb = np.ctypeslib.as_array(b.values, (32,))
        assert a.x0 == b.x0 and a.xn == b.xn
        assert np.max(np.abs(va - vb)) <= 1e-12 * np.max(np.abs(vb)), name
    L.comdgb_cheb_free(cg_cheb)


def test_gpu_fitted_cheby_force(oracle):
    """EAM Chebyshev with the series fitted on the GPU instead of the host."""
    c = Case(oracle, cg.POT_EAM_CHEBY)
    try:
        c.oracle_force()
        d = c.device(cg.PREC_FP64, cheby_from_host=False)
        e, _ = d.force()
        d.download(c.s)
        d.close()
        cmp = compare_forces(c.s, c.o)
        assert cmp["f_max_rel"] < 1e-10, cmp
        assert abs(e - c.o.contents.e) <= 1e-11 * abs(c.o.contents.e)
    finally:
        c.close()


def test_put_atoms_bitexact(oracle):
    """Device counting-sort binning equals n sequential putAtomInBox calls."""
    L = cg.load()
    pot = cg.eam_potential("cu")
    s = cg.fcc(6, 6, 6, 3.615, 1.0, 1.0, pot)
    v = slot_views(s)
    m = v["natoms"].sum()
    rng = np.random.default_rng(3)
    # world coordinates of the lattice atoms, shuffled ids, some outside [0, L)
    dc = v["dcenter"]
    occ = np.arange(64)[None, :] < v["natoms"][:, None]
    boxes = np.nonzero(occ)[0]
    xyz = v["r"][occ.reshape(-1)] + dc[boxes]
    xyz += rng.normal(scale=0.2, size=xyz.shape)
    order = rng.permutation(m)
    xyz = np.ascontiguousarray(xyz[order])
    pxyz = np.ascontiguousarray(rng.normal(size=xyz.shape))
    ids = np.ascontiguousarray(np.arange(m, dtype=np.int32)[::-1])
    types = np.ones(m, dtype=np.int32)
    masses = np.full(m, 63.55)
    o2 = oracle.clone(s)
    # empty both
    for sim in (s, o2):
        vv = slot_views(sim)
        vv["natoms"][:] = 0
        sim.contents.ntot = 0
    for t in range(m):
        assert oracle.lib.orc_put_atom(o2, int(ids[t]), 1, 63.55, *xyz[t], *pxyz[t]) == 0
    rc = L.comdgb_put_atoms(s, m, xyz.ctypes.data, pxyz.ctypes.data, ids.ctypes.data,
                            types.ctypes.data, masses.ctypes.data, 0)
    assert rc == 0, cg.lib.last_error()
    assert s.contents.ntot == m
    assert slots_equal(s, o2)
    cg.free_host(s)
    oracle.free(o2)


def test_dropin_force_and_steps(oracle):
    """attach + pot->force = comdgb_force + comdgb_nTimeSteps on a host simflat_t."""
    L = cg.load()
    c = Case(oracle, cg.POT_EAM_CHEBY)
    try:
        o = cg.opts(cg.POT_EAM_CHEBY, cg.PREC_FP64, cheby_from_host=True)
        assert L.comdgb_attach(c.s, C.byref(o)) == 0, cg.lib.last_error()
        assert L.comdgb_force(C.cast(c.s, C.c_void_p)) == 0
        c.oracle_force()
        cmp = compare_forces(c.s, c.o)
        assert cmp["f_max_rel"] < FP64_F_TOL
        assert abs(c.s.contents.e - c.o.contents.e) <= FP64_E_TOL * abs(c.o.contents.e)
        e = L.comdgb_nTimeSteps(5, c.s, 1e-15)
        assert c.oracle.steps(c.o, 5, 1e-15, c.kind) == 0
        assert abs(e - c.o.contents.e) <= 1e-10 * abs(c.o.contents.e)
        assert layout_equal(c.s, c.o)
        assert L.comdgb_detach(c.s) == 0
    finally:
        c.close()


@pytest.mark.parametrize("precision", [cg.PREC_FP64, cg.PREC_MIXED])
def test_persistent_lists_match_per_step_lists(oracle, precision):
    """Lists kept across steps (skin) give the same forces as lists rebuilt
    every step, and trajectories with several rebuilds track the oracle.
    The same pairs: equal pair counts.  FP64 sums in the same order (energy
    to 1e-12); mixed precision's force-order lists come in sub-cell order,
    so its compensated FP32 per-atom sums may differ in the last bits
    (energy to 1e-8)."""
    c = Case(oracle, cg.POT_EAM_CHEBY, n=(8, 8, 8), temp=1200.0, amp=0.05)
    try:
        dp = cg.DeviceSim(c.s, cg.opts(cg.POT_EAM_CHEBY, precision, cheby_from_host=True,
                                       skin=0.1))
        ds = cg.DeviceSim(c.s, cg.opts(cg.POT_EAM_CHEBY, precision, cheby_from_host=True,
                                       per_step_lists=True))
        assert dp.list_info()[0] and not ds.list_info()[0]
        ep, _ = dp.force()
        es, _ = ds.force()
        assert dp.pair_count() == ds.pair_count()
        tol = 1e-12 if precision == cg.PREC_FP64 else 1e-8
        assert abs(ep - es) <= tol * abs(es)
        n = 40
        ep, _ = dp.steps(n, 1e-15)
        es, _ = ds.steps(n, 1e-15)
        persistent, skin, builds = dp.list_info()
        assert builds >= 3, builds  # 1200 K with a 0.1 A skin rebuilds several times
        assert dp.pair_count() == ds.pair_count()
        if precision == cg.PREC_FP64:
            assert c.oracle.steps(c.o, n, 1e-15, c.kind) == 0
            assert abs(ep - c.o.contents.e) <= 1e-10 * abs(c.o.contents.e)
            dp.download(c.s)
            assert layout_equal(c.s, c.o)
        else:
            assert abs(ep - es) <= 1e-7 * abs(es)
        dp.close()
        ds.close()
    finally:
        c.close()



@pytest.mark.parametrize("n", [1, 2, 3, 7])
def test_step_sequences_match_single_steps(oracle, n):
    """In force order a sequence of n steps makes every step's velocity step
    and position half steps inside the force pass before it, except the last
    step's, which the closing part makes (the ST_FUSE flag the host sets and
    clears).  n steps in one call against n calls of one step (where no
    force pass makes an update) agree up to the roundings of adding the two
    half steps at once: a misplaced update would be off by half a step."""
    c = Case(oracle, cg.POT_EAM_CHEBY, n=(8, 8, 8), temp=900.0, amp=0.05)
    try:
        o = cg.opts(cg.POT_EAM_CHEBY, cg.PREC_MIXED, cheby_from_host=True)
        res = []
        for calls, s in ((1, c.s), (n, c.o)):
            d = cg.DeviceSim(s, o)
            try:
                assert d.list_info()[0]
                for _ in range(calls):
                    e, _ = d.steps(n // calls, 1e-15)
                d.download(s)
            finally:
                d.close()
            res.append((e, world_by_id(s), by_id(s, "p")[:, :3].copy()))
        (e0, w0, p0), (e1, w1, p1) = res
        assert abs(e1 - e0) <= 1e-10 * abs(e0), (e0, e1)
        dw = w1 - w0
        L = np.array(list(c.s.contents.bounds))
        dw -= L * np.round(dw / L)
        assert np.abs(dw).max() < 1e-9
        assert rel_rms(p1, p0) < 1e-9
    finally:
        c.close()


@pytest.mark.parametrize("kw", [dict(periodic=False), dict(n=(4, 4, 4)), dict(n=(2, 5, 4))],
                         ids=["nonperiodic", "two-box-grid", "mixed-grid"])
def test_mixed_without_force_order(oracle, kw):
    """mixed precision where force order does not apply (non-periodic, or
    fewer than 3 boxes on an axis): per-step FP32 lists; forces and a
    10-step trajectory against the FP64 oracle"""
    c = Case(oracle, cg.POT_EAM_CHEBY, temp=600.0, amp=0.05, **kw)
    try:
        d = c.device(cg.PREC_MIXED)
        try:
            assert not d.list_info()[0] or kw.get("periodic", True)
            d.force()
            d.download(c.s)
            c.oracle_force()
            cmp = compare_forces(c.s, c.o)
            assert cmp["f_rel_rms"] < MIXED_F_RMS_TOL, cmp
            e, _ = d.steps(10, 1e-15)
        finally:
            d.close()
        assert c.oracle.steps(c.o, 10, 1e-15, c.kind) == 0
        assert abs(e - c.o.contents.e) / c.s.contents.ntot < 1e-7
    finally:
        c.close()


def test_lj_mixed_trajectory(oracle):
    """LJ in force order over 50 steps (the reference's sign, short enough to
    stay near the lattice): energy per atom within 1e-6 of the FP64 oracle"""
    c = Case(oracle, cg.POT_LJ, n=(8, 8, 8), disp=cg.DISP_UNIFORM, amp=0.01 * 2.315, temp=0.0)
    try:
        d = c.device(cg.PREC_MIXED)
        try:
            assert d.list_info()[0]
            e, _ = d.steps(50, 1e-15)
        finally:
            d.close()
        assert c.oracle.steps(c.o, 50, 1e-15, c.kind) == 0
        assert abs(e - c.o.contents.e) / c.s.contents.ntot < 1e-6, (e, c.o.contents.e)
    finally:
        c.close()


@pytest.mark.parametrize("periodic", [True, False], ids=["force-order", "nonperiodic"])
def test_merged_rebox_matches_two_reboxes(oracle, periodic):
    """Mixed precision reboxes once per step inside a sequence of steps (the
    closing position half step of a step and the opening one of the next run
    back to back).  Against the reference's two reboxes per step the
    trajectory differs only by roundings: energy within 1e-9, world
    positions within 1e-8 A and momenta within 1e-9 by id; every atom ends in
    its box, so the oracle's reBoxAll moves nothing."""
    c = Case(oracle, cg.POT_EAM_CHEBY, n=(8, 8, 8), temp=1200.0, amp=0.05, periodic=periodic)
    try:
        res = []
        for merge, s in ((False, c.s), (True, c.o)):
            d = cg.DeviceSim(s, cg.opts(cg.POT_EAM_CHEBY, cg.PREC_MIXED, periodic,
                                        cheby_from_host=True))
            try:
                d.set_merge_rebox(merge)
                e, _ = d.steps(20, 1e-15)
                d.download(s)
            finally:
                d.close()
            o2 = oracle.clone(s)
            try:
                assert oracle.rebox(o2) == 0
                assert slots_equal(s, o2)
            finally:
                oracle.free(o2)
            res.append((e, world_by_id(s), by_id(s, "p")[:, :3].copy()))
        (e0, w0, p0), (e1, w1, p1) = res
        assert abs(e1 - e0) <= 1e-9 * abs(e0), (e0, e1)
        dw = w1 - w0
        if periodic:
            L = np.array(list(c.s.contents.bounds))
            dw -= L * np.round(dw / L)
        assert np.abs(dw).max() < 1e-8
        assert rel_rms(p1, p0) < 1e-9
    finally:
        c.close()


def test_merge_rebox_is_mixed_only(oracle):
    c = Case(oracle, cg.POT_EAM_TABLE, n=(6, 6, 6))
    try:
        d = c.device(cg.PREC_FP64)
        try:
            with pytest.raises(cg.ComdgbError):
                d.set_merge_rebox(True)
            d.set_merge_rebox(False)
        finally:
            d.close()
    finally:
        c.close()
