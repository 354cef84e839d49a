"""The parity configurations beside the headline, at their full sizes.

C1 -- the reference's default LJ run: FCC 20^3 (32,000 atoms), lattice
3.615 A, sigma 2.315 A, epsilon 0.167 eV, cutoff 2.5 sigma, mass 63.55,
box factor 1, seeded uniform +-0.01 sigma displacements, zero momenta,
dt = 1 fs.  The reference's LJ forces carry the physical sign while its
integrator subtracts them (ljForce.c:205-209, timestep.c:62-74), so the
trajectory runs away from the lattice and any two implementations part
exponentially: the comparison is step 0 (forces, energies, the scalar
stress and the virial tensor) and the first 10 steps.  The 100-step run does
not finish in the reference: the lattice collapses and the reference aborts
with "Increase maxatoms" (-11) at step 76 (its own build, run here).  By
then the trajectories have parted completely, so the library must stop
within three steps of the oracle, by a box overflow (-11) or by the
infinite energy of a coincident pair (-35) -- the same collapse.

C2 -- EAM Cu by table lookup, FP64: FCC 40^3 (256,000 atoms), box factor 1,
Gaussian displacements sigma 0.05 A, momenta at 600 K, dt = 1 fs: step 0
and 10 steps against the oracle, then the total energy over 1000 steps
(drift within 1e-4 eV/atom, the target of the mixed-precision step; FP64
sits far below it).
"""
import numpy as np
import pytest

import comd_gb300 as cg
from comd_gb300.abi import by_id
from helpers import Case, compare_forces, layout_equal, rel_rms

SIGMA = 2.315


def c1(oracle):
    return Case(oracle, cg.POT_LJ, n=(20, 20, 20), disp=cg.DISP_UNIFORM, amp=0.01 * SIGMA,
                temp=0.0)


def c2(oracle):
    return Case(oracle, cg.POT_EAM_TABLE, n=(40, 40, 40), disp=cg.DISP_GAUSSIAN, amp=0.05,
                temp=600.0)


def check_step0(c, d):
    """FP64 force call on the device against the oracle: per-atom forces and
    energies, totals, the reference's scalar stress and the virial tensor"""
    e, st = d.force()
    w, k, _ = d.virial()
    d.download(c.s)
    c.oracle_force()
    cmp = compare_forces(c.s, c.o)
    assert cmp["f_max_rel"] < 1e-10, cmp
    assert cmp["e_max_rel"] < 1e-10, cmp
    assert abs(e - c.o.contents.e) <= 1e-12 * abs(c.o.contents.e)
    assert abs(st - c.o.contents.stress) <= 1e-10 * abs(c.o.contents.stress)
    wo, ko, _ = c.oracle.virial(c.o, c.kind)
    assert np.abs(w - wo).max() <= 1e-11 * np.abs(wo).max()
    assert np.abs(k - ko).max() <= 1e-13 * max(np.abs(ko).max(), 1e-300)


def check_steps(c, d, n=10):
    e, _ = d.steps(n, 1e-15)
    d.download(c.s)
    assert c.oracle.steps(c.o, n, 1e-15, c.kind) == 0
    assert abs(e - c.o.contents.e) <= 1e-10 * abs(c.o.contents.e), (e, c.o.contents.e)
    assert layout_equal(c.s, c.o)
    assert np.abs(by_id(c.s, "r") - by_id(c.o, "r")).max() < 1e-9
    assert rel_rms(by_id(c.s, "p"), by_id(c.o, "p")) < 1e-8


@pytest.mark.gpu
def test_c1_lj_default_run(oracle):
    c = c1(oracle)
    try:
        assert c.s.contents.ntot == 32000
        d = c.device()
        try:
            check_step0(c, d)
            check_steps(c, d, 10)
            stop_gpu = None
            for k in range(11, 101):
                try:
                    d.steps(1, 1e-15)
                except cg.ComdgbError as e:
                    assert e.code in (-11, -35), e
                    stop_gpu = k
                    break
        finally:
            d.close()
        stop_oracle = None
        for k in range(11, 101):
            rc = c.oracle.steps(c.o, 1, 1e-15, c.kind)
            if rc:
                assert rc == -11
                stop_oracle = k
                break
        assert stop_oracle is not None and stop_gpu is not None
        assert abs(stop_gpu - stop_oracle) <= 3, (stop_gpu, stop_oracle)
    finally:
        c.close()


@pytest.mark.gpu
def test_c1_lj_mixed_force_error(oracle):
    c = c1(oracle)
    try:
        fs = []
        for prec in (cg.PREC_FP64, cg.PREC_MIXED):
            d = c.device(prec)
            try:
                d.force()
                d.download(c.s)
            finally:
                d.close()
            fs.append(by_id(c.s, "f")[:, :3].copy())
        assert rel_rms(fs[1], fs[0]) < 1e-5
    finally:
        c.close()


@pytest.mark.gpu
def test_c2_eam_table_fp64(oracle):
    c = c2(oracle)
    try:
        n = c.s.contents.ntot
        assert n == 256000
        d = c.device()
        try:
            check_step0(c, d)
            check_steps(c, d, 10)
            e0, _ = d.force()
            h0 = e0 + d.kinetic()
            hs = []
            for _ in range(10):
                e, _ = d.steps(99, 1e-15)  # with the 10 above and the force calls: 1000
                hs.append(e + d.kinetic())
        finally:
            d.close()
        drift = max(abs(h - h0) for h in hs) / n
        assert drift < 1e-4 * cg.lib.EV_TO_HA, drift
    finally:
        c.close()


@pytest.mark.gpu
def test_c2_eam_table_mixed(oracle):
    """the same lattice in mixed precision: force error against FP64 and the
    1000-step drift"""
    c = c2(oracle)
    try:
        n = c.s.contents.ntot
        fs = []
        for prec in (cg.PREC_FP64, cg.PREC_MIXED):
            d = c.device(prec)
            try:
                d.force()
                d.download(c.s)
            finally:
                d.close()
            fs.append(by_id(c.s, "f")[:, :3].copy())
        assert rel_rms(fs[1], fs[0]) < 1e-5
        d = c.device(cg.PREC_MIXED)
        try:
            e0, _ = d.force()
            h0 = e0 + d.kinetic()
            hs = []
            for _ in range(10):
                e, _ = d.steps(100, 1e-15)
                hs.append(e + d.kinetic())
        finally:
            d.close()
        drift = max(abs(h - h0) for h in hs) / n
        assert drift < 1e-4 * cg.lib.EV_TO_HA, drift
    finally:
        c.close()
