"""The batch autotuner (comdgb_batch_autotune) and the host rebinning it uses
(comdgb_rebin_host).

CPU: a lattice built at box factor 1.0 and rebinned at 1.25 equals the same
lattice built at 1.25 directly (occupancy and ids exactly; positions to FP64
rounding of box corner + r), and a box factor that would put more than 64
atoms in a box is refused with COMDGB_ERR_MAXATOMS.

GPU: on four uneven replicas the tuner returns a choice among its
candidates, writes it to the cache file, and a second call returns the same
choice from the cache without timing; the chosen launch shapes leave the
batch's results unchanged bit for bit.
"""
import os

import numpy as np
import pytest

import comd_gb300 as cg
from comd_gb300.abi import by_id, slot_views
from helpers import world_by_id

REPLICAS = [(6, 11, 300.0), (7, 12, 900.0), (8, 13, 600.0), (6, 14, 1200.0)]


def test_rebin_host_equals_direct_lattice():
    pot = cg.eam_potential("cu")
    lat = pot.ptr.contents.lat
    a = cg.fcc(9, 8, 7, lat, 1.05, 1.0, pot)
    direct = cg.fcc(9, 8, 7, lat, 1.05, 1.25, pot)
    cg.seed(a, 5, cg.DISP_NONE, 0.0, 600.0, pot.ptr.contents.mass)
    cg.seed(direct, 5, cg.DISP_NONE, 0.0, 600.0, pot.ptr.contents.mass)
    b = cg.rebin_host(a, 1.25)
    try:
        assert list(b.contents.nbx) == list(direct.contents.nbx)
        vb, vd = slot_views(b), slot_views(direct)
        assert np.array_equal(vb["natoms"], vd["natoms"])
        occ = np.arange(64)[None, :] < vd["natoms"][:, None]
        assert np.array_equal(vb["id"][occ.reshape(-1)], vd["id"][occ.reshape(-1)])
        assert np.max(np.abs(world_by_id(b) - world_by_id(direct))) < 1e-12
        assert np.array_equal(by_id(b, "p"), by_id(a, "p"))
        with pytest.raises(cg.ComdgbError) as e:
            cg.rebin_host(a, 2.5)  # boxes of more than 64 atoms
        assert e.value.code == cg.ERR_MAXATOMS
    finally:
        for s in (a, b, direct):
            cg.free_host(s)


def _replicas(pot):
    sims = []
    for n, seed, temp in REPLICAS:
        s = cg.fcc(n, n, n, pot.ptr.contents.lat, 1.0, 1.0, pot)
        cg.seed(s, seed, cg.DISP_GAUSSIAN, 0.03, temp, pot.ptr.contents.mass)
        sims.append(s)
    return sims


@pytest.mark.gpu
def test_autotune_choice_cache_and_results(tmp_path):
    pot = cg.eam_potential("cu")
    o = cg.opts(cg.POT_EAM_CHEBY, cg.PREC_MIXED, True)
    sims = _replicas(pot)
    cache = str(tmp_path / "tune.cache")
    bfs, skins = (1.0, 1.2), (0.3, 0.5)
    try:
        t = cg.batch_autotune(sims, o, bfs, skins, steps=5, cache_path=cache)
        assert not t.from_cache
        assert t.box_factor in bfs and t.skin in skins
        assert t.build_threads in (64, 128, 256) and t.build_atoms in (2, 4, 8)
        assert t.pass2_threads in (128, 256, 512)
        assert t.ms_per_step > 0
        assert os.path.exists(cache) and len(open(cache).read().splitlines()) == 1
        t2 = cg.batch_autotune(sims, o, bfs, skins, steps=5, cache_path=cache)
        assert t2.from_cache
        for k in ("box_factor", "skin", "build_threads", "build_atoms", "pass2_threads"):
            assert getattr(t2, k) == getattr(t, k), k
        # other candidates: another key, timed again
        t3 = cg.batch_autotune(sims, o, (1.0,), (0.5,), steps=5, cache_path=cache)
        assert not t3.from_cache and t3.box_factor == 1.0 and t3.skin == 0.5
        # the tuned launch shapes change no result
        energies = []
        for tune in (None, t):
            b = cg.Batch(sims, o)
            try:
                if tune is not None:
                    b.apply_tune(tune)
                b.steps(8)
                energies.append(b.energies()[0])
            finally:
                b.close()
        assert np.array_equal(energies[0], energies[1])
    finally:
        for s in sims:
            cg.free_host(s)
