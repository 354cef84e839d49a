"""The neighbour-list overflow fallback.

An atom whose neighbour count exceeds the list capacity is computed by
scanning its 27 neighbour boxes instead of its list (the reference's own
loop, eam.c:484-549 and :595-653).  Capping the capacity below the real
neighbour count (comdgb_sim_set_list_capacity) sends every atom (a capacity
of 8), or the atoms with more than the 54 neighbours that a perfect lattice
has within the list cutoff (a capacity of 54), down that path:

* mixed precision, force order: a 40-step sequence across list rebuilds
  must give the trajectory of the uncapped run up to roundings.  Between
  rebuilds the FP32 slot copy of the positions, which the scan reads, has
  to be current.  Atoms are not reboxed between rebuilds; the lattice here
  has the largest skin the library allows (box width minus cutoff), so
  atoms that moved up to skin/2 outside their boxes keep every in-cutoff
  pair within adjacent boxes only just.  The final force call is checked
  against the FP64 oracle on the same positions.
* FP64, id-keyed persistent lists: 10 steps equal the oracle's trajectory
  to the FP64 tolerances of the other trajectory tests.

Tolerances: mixed, capped vs uncapped after 40 steps, positions 1e-5 A and
energy 1e-8 Ha per atom; force call vs the oracle, relative RMS 1e-5.  FP64
vs the oracle after 10 steps: energy 1e-10 relative, positions 1e-9 A.
"""
import numpy as np
import pytest

import comd_gb300 as cg
from comd_gb300.abi import by_id
from helpers import Case, layout_equal, rel_rms, world_by_id

pytestmark = pytest.mark.gpu


def _mixed(c, cap, skin=0.5):
    d = cg.DeviceSim(c.s, cg.opts(cg.POT_EAM_CHEBY, cg.PREC_MIXED, skin=skin,
                                  cheby_from_host=True))
    persistent, used_skin, _ = d.list_info()
    assert persistent and used_skin < skin  # capped at box width minus cutoff
    if cap:
        d.set_list_capacity(cap)
    return d


def _min_image(a, b, bounds):
    d = a - b
    return d - np.round(d / bounds) * bounds


@pytest.mark.parametrize("cap", [8, 54])
def test_mixed_overflow_trajectory(oracle, cap):
    # 12^3 cells, box factor 1: 8 boxes of 5.4225 A per axis against a
    # 4.961 A cutoff, skin 0.4615 A (capped at box width minus cutoff); 600 K
    # so that lists are rebuilt within the sequence
    c = Case(oracle, cg.POT_EAM_CHEBY, n=(12, 12, 12), bf=1.0, temp=600.0, amp=0.05, seed=31)
    try:
        assert list(c.s.contents.nbx) == [8, 8, 8]
        bounds = np.array(c.s.contents.bounds[:3])
        ref = _mixed(c, 0)
        capped = _mixed(c, cap)
        try:
            e_ref, _ = ref.steps(40, 1e-15)
            e_cap, _ = capped.steps(40, 1e-15)
            builds = capped.list_info()[2]
            s_ref = cg.fcc(12, 12, 12, c.pot.ptr.contents.lat, 1.0, 1.0, c.pot)
            try:
                ref.download(s_ref)
                capped.download(c.s)
                dr = _min_image(world_by_id(c.s), world_by_id(s_ref), bounds)
            finally:
                cg.free_host(s_ref)
        finally:
            ref.close()
            capped.close()
        n = c.s.contents.ntot
        print(f"cap {cap}: builds {builds}, max |dr| {np.abs(dr).max():.3e} A, "
              f"dE/N {abs(e_cap - e_ref) / n:.3e}")
        assert builds >= 2, "the sequence must cross a list rebuild"
        assert np.abs(dr).max() < 1e-5
        assert abs(e_cap - e_ref) / n < 1e-8
        # the final force call against the oracle on the same positions
        o2 = oracle.clone(c.s)
        try:
            assert oracle.force(o2, c.kind) == 0
            err = rel_rms(by_id(c.s, "f")[:, :3], by_id(o2, "f")[:, :3])
            assert err < 1e-5, err
            assert abs(e_cap - o2.contents.e) / n < 1e-7
        finally:
            oracle.free(o2)
    finally:
        c.close()


def test_fp64_idkeyed_overflow_vs_oracle(oracle):
    c = Case(oracle, cg.POT_EAM_CHEBY, n=(8, 8, 8), temp=600.0, amp=0.05, seed=32)
    try:
        d = cg.DeviceSim(c.s, cg.opts(cg.POT_EAM_CHEBY, cg.PREC_FP64, cheby_from_host=True))
        try:
            assert d.list_info()[0]
            # thermal atoms with more than the 54 lattice neighbours overflow
            d.set_list_capacity(54)
            e, _ = d.steps(10, 1e-15)
            d.download(c.s)
        finally:
            d.close()
        assert c.oracle.steps(c.o, 10, 1e-15, c.kind) == 0
        eo = c.o.contents.e
        assert abs(e - eo) <= 1e-10 * abs(eo), (e, eo)
        assert layout_equal(c.s, c.o)
        assert np.max(np.abs(by_id(c.s, "r") - by_id(c.o, "r"))) < 1e-9
    finally:
        c.close()


def test_list_capacity_bounds():
    pot = cg.eam_potential("cu")
    s = cg.fcc(6, 6, 6, pot.ptr.contents.lat, 1.0, 1.0, pot)
    try:
        d = cg.DeviceSim(s, cg.opts(cg.POT_EAM_CHEBY, cg.PREC_MIXED))
        try:
            with pytest.raises(cg.ComdgbError):
                d.set_list_capacity(100000)
            with pytest.raises(cg.ComdgbError):
                d.set_list_capacity(-2)
            d.set_list_capacity(0)
        finally:
            d.close()
    finally:
        cg.free_host(s)
