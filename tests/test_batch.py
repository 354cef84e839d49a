"""Batched replicas: several independent simulations of uneven sizes advanced
by one set of launches (comdgb_batch_*).  Each replica must come out exactly
as if it had run alone: with per-step lists the FP64 trajectories, slot
layouts and energies are bit-identical to single-simulation runs; with the
default skin lists (one rebuild flag for the whole batch) mixed precision
agrees to rounding."""
import numpy as np
import pytest

import comd_gb300 as cg
from helpers import slots_equal

REPLICAS = [((5, 5, 5), 1.0, 11, 300.0), ((7, 6, 5), 1.0, 12, 900.0), ((6, 6, 6), 1.25, 13, 600.0),
            ((4, 5, 6), 1.0, 14, 1200.0)]


def make_replicas(pot):
    sims = []
    for (n, bf, seed, temp) in REPLICAS:
        s = cg.fcc(n[0], n[1], n[2], pot.ptr.contents.lat, 1.0, bf, pot)
        cg.seed(s, seed, cg.DISP_GAUSSIAN, 0.03, temp, pot.ptr.contents.mass)
        sims.append(s)
    return sims


def single_run(s, o, nsteps):
    d = cg.DeviceSim(s, o)
    try:
        e = d.steps(nsteps)[0]
        d.download(s)
    finally:
        d.close()
    return e


@pytest.mark.gpu
def test_batch_fp64_bit_identical_to_single_runs():
    pot = cg.eam_potential("cu")
    o = cg.opts(cg.POT_EAM_CHEBY, cg.PREC_FP64, True, per_step_lists=True)
    batch_sims, single_sims = make_replicas(pot), make_replicas(pot)
    try:
        b = cg.Batch(batch_sims, o)
        try:
            assert b.n == len(REPLICAS)
            b.steps(10)
            e_b, _ = b.energies()
            for r, s in enumerate(batch_sims):
                b.download_rep(r, s)
        finally:
            b.close()
        for r, s in enumerate(single_sims):
            e = single_run(s, o, 10)
            assert slots_equal(batch_sims[r], s, ("id", "iType", "mass", "r", "p")), r
            assert abs(e_b[r] - e) <= 1e-12 * abs(e), r
    finally:
        for s in batch_sims + single_sims:
            cg.free_host(s)


@pytest.mark.gpu
def test_batch_mixed_matches_single_runs():
    pot = cg.eam_potential("cu")
    o = cg.opts(cg.POT_EAM_CHEBY, cg.PREC_MIXED, True)
    batch_sims, single_sims = make_replicas(pot), make_replicas(pot)
    try:
        b = cg.Batch(batch_sims, o)
        try:
            b.steps(20)
            e_b, st_b = b.energies()
            for r, s in enumerate(batch_sims):
                b.download_rep(r, s)
        finally:
            b.close()
        for r, s in enumerate(single_sims):
            e = single_run(s, o, 20)
            assert abs(e_b[r] - e) <= 1e-7 * abs(e), (r, e_b[r], e)
            assert np.isfinite(st_b[r])
    finally:
        for s in batch_sims + single_sims:
            cg.free_host(s)


@pytest.mark.gpu
def test_merged_step_paths_agree():
    """mixed precision with the rebox merged: replays of the step parts, the
    n steps captured as one graph and the timed run give the same state bit
    for bit (single simulation and batch)"""
    pot = cg.eam_potential("cu")
    o = cg.opts(cg.POT_EAM_CHEBY, cg.PREC_MIXED, True)
    sims = [make_replicas(pot) for _ in range(3)]
    try:
        devs = [cg.DeviceSim(s[0], o) for s in sims]
        try:
            e0 = devs[0].steps(12)[0]
            devs[1].graph_steps(12)
            e1 = devs[1].energy()[0]
            step_ms, span, groups = devs[2].timed_steps(12)
            e2 = devs[2].energy()[0]
            per_step = devs[0].graph_kernels()[0]
            assert devs[0].step_launches(12) - devs[0].step_launches(11) == per_step > 0
            for d, s in zip(devs, sims):
                d.download(s[0])
        finally:
            for d in devs:
                d.close()
        assert e0 == e1 == e2
        assert slots_equal(sims[0][0], sims[1][0]) and slots_equal(sims[0][0], sims[2][0])
        assert len(step_ms) == 12 and span >= sum(step_ms) * 0.999
        # merged groups; in force order the rebuild section is one conditional node
        # and the force pass makes the step's velocity and position update
        assert set(groups) in ({"advance_velocity_positions+classify", "rebin_plan_apply",
                                "compact_atoms", "nbr_build", "force_pass1", "force_pass2"},
                               {"rebuild_if_due", "force_pass1",
                                "force_pass2+advance_velocity_positions"})
        ba, bb = cg.Batch(sims[0][1:], o), cg.Batch(sims[1][1:], o)
        try:
            ba.steps(8)
            bb.graph_steps(8)
            assert np.array_equal(ba.energies()[0], bb.energies()[0])
        finally:
            ba.close()
            bb.close()
    finally:
        for s in sims:
            for x in s:
                cg.free_host(x)


@pytest.mark.gpu
def test_graph_steps_loop_equals_step_replays():
    """n steps captured as one graph give the same FP64 state as n replays of
    the one-step graph (single simulation and batch)"""
    pot = cg.eam_potential("cu")
    o = cg.opts(cg.POT_EAM_CHEBY, cg.PREC_FP64, True, per_step_lists=True)
    a, b = make_replicas(pot), make_replicas(pot)
    try:
        da, db = cg.DeviceSim(a[0], o), cg.DeviceSim(b[0], o)
        try:
            ea = da.steps(12)[0]
            ms = db.graph_steps(12)
            eb = db.energy()[0]
            da.download(a[0])
            db.download(b[0])
        finally:
            da.close()
            db.close()
        assert ms > 0 and ea == eb
        assert slots_equal(a[0], b[0])
        ba, bb = cg.Batch(a[1:], o), cg.Batch(b[1:], o)
        try:
            ba.steps(8)
            bb.graph_steps(8)
            assert np.array_equal(ba.energies()[0], bb.energies()[0])
        finally:
            ba.close()
            bb.close()
    finally:
        for s in a + b:
            cg.free_host(s)


@pytest.mark.gpu
def test_launch_shapes_do_not_change_results():
    """every launch shape of the force-order kernels gives the same state,
    bit for bit (lists and per-atom sums keep their order), single and batch"""
    pot = cg.eam_potential("cu")
    o = cg.opts(cg.POT_EAM_CHEBY, cg.PREC_MIXED, True)
    ref = make_replicas(pot)
    try:
        d = cg.DeviceSim(ref[0], o)
        try:
            e_ref = d.steps(12)[0]
            d.download(ref[0])
        finally:
            d.close()
        b = cg.Batch(ref[1:], o)
        try:
            b.steps(12)
            eb_ref = b.energies()[0]
        finally:
            b.close()
        for shape in [(64, 2, 128), (256, 8, 512), (128, 4, 256), (64, 8, 256)]:
            sims = make_replicas(pot)
            try:
                d = cg.DeviceSim(sims[0], o)
                try:
                    assert d.list_info()[0]
                    d.set_launch(*shape)
                    e = d.steps(12)[0]
                    d.download(sims[0])
                finally:
                    d.close()
                assert e == e_ref, shape
                assert slots_equal(sims[0], ref[0], ("id", "r", "p")), shape
                b = cg.Batch(sims[1:], o)
                try:
                    b.set_launch(*shape)
                    b.steps(12)
                    assert np.array_equal(b.energies()[0], eb_ref), shape
                finally:
                    b.close()
            finally:
                for s in sims:
                    cg.free_host(s)
        with pytest.raises(cg.ComdgbError):
            d = cg.DeviceSim(ref[0], o)
            try:
                d.set_launch(96, 4, 256)
            finally:
                d.close()
    finally:
        for s in ref:
            cg.free_host(s)
