"""Virial tensor, kinetic tensor and per-atom stress (comdgb_sim_virial,
comdgb_sim_atom_stress), next to the reference's scalar stress.

The reference has no tensor, so the oracle's (oracle/virial_oracle.c) is
pinned by physics against the reference's own energies and forces:
  * W_aa = -dU/d(eps_aa) under a homogeneous strain of box and positions
    (central differences of the oracle energy, which equals the reference's
    bit for bit; EAM Chebyshev and LJ, whose forces are exact gradients);
  * W = sum_i x_i (x) F_i for a non-periodic system (all three potentials;
    the table potential's forces are not exact gradients of its energy, the
    interpolation's derivative being its own formula, eam.c:401-434).
The GPU tensors are then checked against the oracle's: FP64 to 1e-12, mixed
precision to 1e-5 of the largest component.  Voigt order xx yy zz yz xz xy.
"""
import ctypes as C

import numpy as np
import pytest

import comd_gb300 as cg
from comd_gb300.abi import occupied_mask, slot_views
from helpers import Case

VOIGT = [(0, 0), (1, 1), (2, 2), (1, 2), (0, 2), (0, 1)]
POTS = [cg.POT_EAM_TABLE, cg.POT_EAM_CHEBY, cg.POT_LJ]


def stretched_case(oracle, potential, **kw):
    """a perturbed, thermal lattice 1 % above its equilibrium spacing, so
    the virial is far from zero"""
    lat = 3.615 * 1.01
    return Case(oracle, potential, n=(6, 6, 6), amp=0.05, temp=600.0, lat=lat, **kw)


def strain_energy(oracle, s, kind, ax, h):
    sc = np.ones(3)
    sc[ax] += h
    t = oracle.strained(s, sc)
    try:
        assert oracle.rebox(t) == 0
        assert oracle.force(t, kind) == 0
        return t.contents.e
    finally:
        oracle.free(t)


def strain_fd(oracle, s, kind, ax, h):
    return -(strain_energy(oracle, s, kind, ax, h) - strain_energy(oracle, s, kind, ax, -h)) / (2 * h)


# ---------------------------------------------------------------- CPU ----

@pytest.mark.parametrize("potential", [cg.POT_EAM_CHEBY, cg.POT_LJ])
def test_oracle_virial_is_the_strain_derivative(oracle, potential):
    """central differences with h = 1e-6 and h/4; a bracket in which a pair
    crosses the cutoff (the energy jumps there: neither potential is shifted
    to zero at rc) shows up as a disagreement between the two and is not
    used"""
    c = stretched_case(oracle, potential)
    try:
        c.oracle_force()
        w, k, _ = oracle.virial(c.o, c.kind)
        scale = np.abs(w).max()
        used = 0
        for ax in range(3):
            fd = strain_fd(oracle, c.o, c.kind, ax, 1e-6)
            fd4 = strain_fd(oracle, c.o, c.kind, ax, 2.5e-7)
            if abs(fd - fd4) > 1e-6 * scale:
                continue
            used += 1
            assert abs(w[ax] - fd) <= 1e-6 * scale, (ax, w[ax], fd)
        assert used >= 2
        assert np.all(k[:3] > 0)
    finally:
        c.close()


@pytest.mark.parametrize("potential", POTS)
def test_oracle_virial_is_the_position_force_moment(oracle, potential):
    """non-periodic: W = sum_i x_i (x) F_i with the reference's forces
    (F = -f for EAM, whose f is +grad U; F = f for LJ)"""
    c = Case(oracle, potential, n=(6, 6, 6), amp=0.05, temp=600.0, periodic=False)
    try:
        c.oracle_force()
        w, k, atoms = oracle.virial(c.o, c.kind, atoms=True)
        v = slot_views(c.o)
        m = occupied_mask(c.o)
        x = (np.repeat(v["dcenter"], 64, axis=0) + v["r"])[m]
        fv = slot_forces(c.o)[m]
        F = -fv if potential != cg.POT_LJ else fv
        mom = np.einsum("ia,ib->ab", x, F)
        ref = np.array([mom[a, b] for a, b in VOIGT])
        scale = np.abs(w).max()
        assert np.abs(w - ref).max() <= 1e-10 * scale, (w, ref)
        # per-atom stresses add up to -(W + K)
        assert np.allclose(atoms.sum(axis=0), -(w + k), rtol=0, atol=1e-12 * np.abs(w + k).max())
        assert np.all(atoms[~m] == 0)
    finally:
        c.close()


def slot_forces(sp):
    """f xyz per slot (the real4 slot array)"""
    s = sp.contents
    ns = s.nboxes * 64
    buf = np.ctypeslib.as_array(C.cast(s.f, C.POINTER(C.c_double)), (ns * 4,))
    return buf.reshape(ns, 4)[:, :3].copy()


# ---------------------------------------------------------------- GPU ----

def device_virial(c, precision, per_step_lists=False):
    d = cg.DeviceSim(c.s, cg.opts(c.potential, precision, c.periodic, cheby_from_host=True,
                                  per_step_lists=per_step_lists))
    try:
        w, k, vol = d.virial()
        a = d.atom_stress()
        return w, k, vol, a
    finally:
        d.close()


@pytest.mark.gpu
@pytest.mark.parametrize("potential", POTS)
@pytest.mark.parametrize("per_step_lists", [False, True])
def test_gpu_virial_fp64_matches_oracle(oracle, potential, per_step_lists):
    c = stretched_case(oracle, potential)
    try:
        c.oracle_force()
        wo, ko, ao = oracle.virial(c.o, c.kind, atoms=True)
        w, k, vol, a = device_virial(c, cg.PREC_FP64, per_step_lists)
        b = c.o.contents.bounds
        assert vol == pytest.approx(b[0] * b[1] * b[2], rel=1e-15)
        assert np.abs(w - wo).max() <= 1e-12 * np.abs(wo).max()
        assert np.abs(k - ko).max() <= 1e-13 * np.abs(ko).max()
        assert np.abs(a - ao).max() <= 1e-11 * np.abs(ao).max()
    finally:
        c.close()


@pytest.mark.gpu
@pytest.mark.parametrize("potential", POTS)
def test_gpu_virial_mixed_matches_fp64(oracle, potential):
    c = stretched_case(oracle, potential)
    try:
        w64, k64, _, a64 = device_virial(c, cg.PREC_FP64)
        w32, k32, _, a32 = device_virial(c, cg.PREC_MIXED)
        assert np.abs(w32 - w64).max() <= 1e-5 * np.abs(w64).max()
        assert np.array_equal(k32, k64)  # momenta are FP64 in both
        err = np.sqrt(((a32 - a64) ** 2).sum() / (a64 ** 2).sum())
        assert err < 1e-5
    finally:
        c.close()


@pytest.mark.gpu
def test_gpu_virial_after_steps_matches_oracle(oracle):
    """after 10 FP64 steps (rebinned layouts are the reference's)"""
    c = stretched_case(oracle, cg.POT_EAM_CHEBY)
    try:
        d = cg.DeviceSim(c.s, cg.opts(c.potential, cg.PREC_FP64, True, cheby_from_host=True))
        try:
            d.steps(10, 1e-15)
            w, k, _ = d.virial()
            a = d.atom_stress()
        finally:
            d.close()
        assert c.oracle.steps(c.o, 10, 1e-15, c.kind) == 0
        wo, ko, ao = oracle.virial(c.o, c.kind, atoms=True)
        assert np.abs(w - wo).max() <= 1e-9 * np.abs(wo).max()
        assert np.abs(k - ko).max() <= 1e-9 * np.abs(ko).max()
        assert np.abs(a - ao).max() <= 1e-8 * np.abs(ao).max()
    finally:
        c.close()


@pytest.mark.gpu
def test_gpu_batch_virial_matches_single_runs():
    from test_batch import make_replicas
    pot = cg.eam_potential("cu")
    o = cg.opts(cg.POT_EAM_CHEBY, cg.PREC_FP64, True, per_step_lists=True)
    bs, ss = make_replicas(pot), make_replicas(pot)
    try:
        b = cg.Batch(bs, o)
        try:
            b.steps(5)
            b.virial()
            got = [b.virial_rep(r) for r in range(b.n)]
            atoms = [b.atom_stress(r) for r in range(b.n)]
        finally:
            b.close()
        for r, s in enumerate(ss):
            d = cg.DeviceSim(s, o)
            try:
                d.steps(5)
                w, k, vol = d.virial()
                a = d.atom_stress()
            finally:
                d.close()
            assert np.abs(got[r][0] - w).max() <= 1e-13 * np.abs(w).max(), r
            assert np.abs(got[r][1] - k).max() <= 1e-13 * np.abs(k).max(), r
            assert got[r][2] == vol
            assert np.abs(atoms[r] - a).max() <= 1e-12 * np.abs(a).max(), r
    finally:
        for s in bs + ss:
            cg.free_host(s)
