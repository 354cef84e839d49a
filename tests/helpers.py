"""Shared builders for the parity tests: seeded inputs made once by the
library's host setup and cloned for the oracle, so both sides start from
identical bytes."""
import hashlib
import json
import os

import numpy as np
import pytest

import comd_gb300 as cg
from comd_gb300.abi import by_id, occupied_mask, slot_views
from oracle import KIND_EAM_CHEBY, KIND_EAM_TABLE, KIND_LJ

EV = cg.lib.EV_TO_HA
# the reference's default LJ run: eps 0.167 eV, sigma 2.315 A, rc 2.5 sigma, Cu mass
LJ_SIGMA, LJ_EPS, LJ_MASS = 2.315, 0.167 * EV, 63.55
LJ_RC = 2.5 * LJ_SIGMA

KIND = {cg.POT_EAM_TABLE: KIND_EAM_TABLE, cg.POT_EAM_CHEBY: KIND_EAM_CHEBY, cg.POT_LJ: KIND_LJ}


class Case:
    """A host simulation from the library's builder plus an oracle clone."""

    def __init__(self, oracle, potential, n=(6, 6, 6), defgrad=1.0, bf=1.0, seed=1,
                 disp=cg.DISP_GAUSSIAN, amp=0.05, temp=600.0, periodic=True, lat=None):
        self.oracle = oracle
        self.potential = potential
        if potential == cg.POT_LJ:
            self.pot = cg.lj_potential(LJ_SIGMA, LJ_EPS, LJ_RC, LJ_MASS)
            lat = lat or 3.615
            mass = LJ_MASS
        else:
            self.pot = cg.eam_potential("cu")
            lat = lat or self.pot.ptr.contents.lat
            mass = self.pot.ptr.contents.mass
        self.s = cg.fcc(n[0], n[1], n[2], lat, defgrad, bf, self.pot)
        cg.seed(self.s, seed, disp, amp, temp, mass)
        self.cheb = None
        if potential == cg.POT_EAM_CHEBY:
            self.cheb = oracle.cheby(self.pot.ptr, 32)
            self.s.contents.ch_pot = self.cheb
        oracle.set_periodic(periodic)
        self.periodic = periodic
        assert oracle.rebox(self.s) == 0
        self.o = oracle.clone(self.s)

    @property
    def kind(self):
        return KIND[self.potential]

    def oracle_force(self):
        assert self.oracle.force(self.o, self.kind) == 0

    def device(self, precision=cg.PREC_FP64, cheby_from_host=True):
        return cg.DeviceSim(self.s, cg.opts(self.potential, precision, self.periodic,
                                             cheby_from_host=cheby_from_host))

    def close(self):
        self.oracle.set_periodic(True)
        cg.free_host(self.s)
        self.oracle.free(self.o)


def rel_rms(a, b):
    return float(np.sqrt(np.mean((a - b) ** 2)) / max(np.sqrt(np.mean(b ** 2)), 1e-300))


def max_rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def compare_forces(sg, so):
    """per-id comparison of f (xyz), per-atom energy, rho, fi."""
    fg, fo = by_id(sg, "f"), by_id(so, "f")
    out = {
        "f_rel_rms": rel_rms(fg[:, :3], fo[:, :3]),
        "f_max_rel": max_rel(fg[:, :3], fo[:, :3]),
        "e_max_rel": max_rel(fg[:, 3], fo[:, 3]),
        "rho_max_rel": max_rel(by_id(sg, "rho"), by_id(so, "rho")),
        "fi_max_rel": max_rel(by_id(sg, "fi"), by_id(so, "fi")),
    }
    return out


def layout_equal(sa, sb):
    va, vb = slot_views(sa), slot_views(sb)
    m = occupied_mask(sa)
    if not np.array_equal(va["natoms"], vb["natoms"]):
        return False
    return bool(np.array_equal(va["id"][m], vb["id"][m]))


def world_by_id(s):
    """world positions by atom id (box centre plus box-relative r)"""
    v = slot_views(s)
    m = occupied_mask(s)
    out = np.empty((s.contents.ntot, 3))
    out[v["id"][m]] = (np.repeat(v["dcenter"], 64, axis=0) + v["r"])[m, :3]
    return out


def slots_equal(sa, sb, fields=("id", "iType", "mass", "r", "p")):
    va, vb = slot_views(sa), slot_views(sb)
    m = occupied_mask(sa)
    if not np.array_equal(va["natoms"], vb["natoms"]):
        return False
    return all(np.array_equal(va[f][m], vb[f][m]) for f in fields)


# ------------------------------------------------ reference fixtures ----

FIX = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                                  "reference_fixtures.json")))


def layout_hash(s):
    """sha256 of the box occupancies and the ids in slot order"""
    v = slot_views(s)
    m = occupied_mask(s)
    h = hashlib.sha256()
    h.update(v["natoms"].astype(np.int32).tobytes())
    h.update(v["id"][m].astype(np.int32).tobytes())
    return h.hexdigest()


def snapshot(s):
    f = by_id(s, "f")
    return {"e": s.contents.e, "stress": s.contents.stress, "ntot": s.contents.ntot,
            "f_first": f[:12], "f_abs_sum": float(np.abs(f[:, :3]).sum()),
            "rho_first": by_id(s, "rho")[:12], "fi_first": by_id(s, "fi")[:12],
            "r_first": by_id(s, "r")[:12], "p_first": by_id(s, "p")[:12],
            "layout": layout_hash(s)}


def match(snap, ref, rtol=1e-12, vrtol=1e-12):
    """a snapshot against a reference fixture: layout exact, energy to rtol,
    the per-atom vectors of the first ids to vrtol (absolute floor 1e-3 of
    that relative bound times the largest entry)"""
    assert snap["ntot"] == ref["ntot"]
    assert snap["layout"] == ref["layout"]
    assert snap["e"] == pytest.approx(ref["e"], rel=rtol)
    assert snap["stress"] == pytest.approx(ref["stress"], rel=1e-10, abs=1e-18)
    scale = max(np.abs(np.array(ref["f_first"])[:, :3]).max(), 1e-12)
    assert np.allclose(snap["f_first"], ref["f_first"], rtol=0, atol=1e-11 * scale)
    assert snap["f_abs_sum"] == pytest.approx(ref["f_abs_sum"], rel=1e-9, abs=1e-12)
    for k in ("rho_first", "fi_first", "r_first", "p_first"):
        r = np.array(ref[k])
        assert np.allclose(snap[k], r, rtol=vrtol, atol=1e-3 * vrtol * np.abs(r).max()), k
