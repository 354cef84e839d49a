"""The drop-in calls on a host simflat_t (comdgb_attach, comdgb_force,
comdgb_nTimeSteps, comdgb_reBoxAll), eager and lazy.

Eager (the default): every call copies the host state up and the results
back.  Lazy: the state stays on the GPU between calls; the host sees e and
stress after each call and the slot arrays after comdgb_sync_to_host (or
comdgb_detach); comdgb_sync_to_device hands host changes to the GPU.  With
per-step FP64 lists the two modes give the same trajectory bit for bit."""
import ctypes as C

import numpy as np
import pytest

import comd_gb300 as cg
from comd_gb300.abi import by_id, slot_views
from helpers import Case, rel_rms, slots_equal, world_by_id


def opts():
    return cg.opts(cg.POT_EAM_CHEBY, cg.PREC_FP64, True, cheby_from_host=True,
                   per_step_lists=True)


@pytest.mark.gpu
def test_lazy_equals_eager(oracle):
    a = Case(oracle, cg.POT_EAM_CHEBY, n=(6, 6, 6), amp=0.05, temp=600.0)
    b = Case(oracle, cg.POT_EAM_CHEBY, n=(6, 6, 6), amp=0.05, temp=600.0)
    L = cg.load()
    L.comdgb_set_lazy.argtypes = [C.c_void_p, C.c_int]
    try:
        r0 = slot_views(a.s)["r"].copy()
        o = opts()
        assert L.comdgb_attach(a.s, C.byref(o)) == 0
        assert L.comdgb_attach(b.s, C.byref(o)) == 0
        try:
            assert L.comdgb_set_lazy(a.s, 1) == 0
            ea = [L.comdgb_nTimeSteps(5, a.s, 1e-15) for _ in range(3)]
            eb = [L.comdgb_nTimeSteps(5, b.s, 1e-15) for _ in range(3)]
            assert ea == eb
            assert a.s.contents.e == b.s.contents.e
            # lazy: the host's arrays are still the initial ones ...
            assert np.array_equal(slot_views(a.s)["r"], r0)
            # ... until they are synced
            assert L.comdgb_sync_to_host(a.s) == 0
            assert slots_equal(a.s, b.s, ("id", "r", "p", "f", "rho", "fi"))
            # host changes reach the device by sync_to_device
            for s in (a.s, b.s):
                slot_views(s)["p"][:] *= 0.5
            assert L.comdgb_sync_to_device(a.s) == 0
            assert L.comdgb_nTimeSteps(3, a.s, 1e-15) == L.comdgb_nTimeSteps(3, b.s, 1e-15)
            assert L.comdgb_force(C.cast(a.s, C.c_void_p)) == 0
            assert L.comdgb_force(C.cast(b.s, C.c_void_p)) == 0
            assert a.s.contents.e == b.s.contents.e
        finally:
            assert L.comdgb_detach(a.s) == 0  # lazy: brings the state home first
            assert L.comdgb_detach(b.s) == 0
        assert slots_equal(a.s, b.s, ("id", "r", "p", "f", "rho", "fi"))
    finally:
        a.close()
        b.close()


@pytest.mark.gpu
def test_eager_force_matches_oracle(oracle):
    """comdgb_force installed as the potential's force pointer computes what
    the reference's computeForce computes (FP64)"""
    c = Case(oracle, cg.POT_EAM_TABLE, n=(6, 6, 6), amp=0.05, temp=600.0)
    L = cg.load()
    try:
        o = cg.opts(cg.POT_EAM_TABLE, cg.PREC_FP64)
        assert L.comdgb_attach(c.s, C.byref(o)) == 0
        try:
            assert L.comdgb_force(C.cast(c.s, C.c_void_p)) == 0
        finally:
            L.comdgb_detach(c.s)
        c.oracle_force()
        assert abs(c.s.contents.e - c.o.contents.e) <= 1e-12 * abs(c.o.contents.e)
        assert abs(c.s.contents.stress - c.o.contents.stress) <= 1e-10 * abs(c.o.contents.stress)
    finally:
        c.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [cg.PREC_FP64, cg.PREC_MIXED])
def test_eager_calls_keep_lists(oracle, precision):
    """Eager calls upload the host state each time; skin lists built by an
    earlier call stay (maps redone, skin test decides), so 4 eager calls of
    5 steps give the same state as 20 steps on a handle, and build the lists
    only when atoms moved, not once per call.  FP64: bit for bit.  Mixed
    precision reboxes once per step inside a call but after the last half
    step of each call, so the states agree to roundings: by atom id,
    energies within 1e-12, world positions within 1e-10 A, momenta and
    forces within 1e-10."""
    a = Case(oracle, cg.POT_EAM_CHEBY, n=(8, 8, 8), amp=0.05, temp=600.0)
    b = Case(oracle, cg.POT_EAM_CHEBY, n=(8, 8, 8), amp=0.05, temp=600.0)
    L = cg.load()
    try:
        o = cg.opts(cg.POT_EAM_CHEBY, precision, True, cheby_from_host=True)
        d = cg.DeviceSim(b.s, o)
        try:
            assert d.list_info()[0]
            eb = d.steps(20, 1e-15)[0]
            d.download(b.s)
        finally:
            d.close()
        assert L.comdgb_attach(a.s, C.byref(o)) == 0
        try:
            for _ in range(4):
                ea = L.comdgb_nTimeSteps(5, a.s, 1e-15)
        finally:
            L.comdgb_detach(a.s)
        if precision == cg.PREC_FP64:
            assert ea == eb
            assert slots_equal(a.s, b.s, ("id", "r", "p", "f", "rho", "fi"))
        else:
            assert abs(ea - eb) <= 1e-12 * abs(eb), (ea, eb)
            dw = world_by_id(a.s) - world_by_id(b.s)
            L = np.array(list(a.s.contents.bounds))
            dw -= L * np.round(dw / L)
            assert np.abs(dw).max() < 1e-10
            for f in ("p", "f"):
                assert rel_rms(by_id(a.s, f)[:, :3], by_id(b.s, f)[:, :3]) < 1e-10, f
    finally:
        a.close()
        b.close()


@pytest.mark.gpu
def test_eager_transfers_move_occupied_slots_only(oracle):
    """An attached simflat_t's arrays are registered; the upload and the
    download of the force results are kernels that read or write only the
    occupied slots.  One eager nTimeSteps call uploads natoms and the state
    of ntot atoms (no f, rho, fi: the call computes them) and downloads
    natoms, the state of ntot atoms (beside the trailing force call) and the
    force results of ntot atoms, byte for byte; the results equal a device
    handle's."""
    a = Case(oracle, cg.POT_EAM_CHEBY, n=(8, 8, 8), amp=0.05, temp=600.0)
    b = Case(oracle, cg.POT_EAM_CHEBY, n=(8, 8, 8), amp=0.05, temp=600.0)
    L = cg.load()
    try:
        o = cg.opts(cg.POT_EAM_CHEBY, cg.PREC_FP64, True, cheby_from_host=True,
                    per_step_lists=True)
        d = cg.DeviceSim(b.s, o)
        try:
            eb = d.steps(3, 1e-15)[0]
            d.download(b.s)
        finally:
            d.close()
        assert L.comdgb_attach(a.s, C.byref(o)) == 0
        try:
            h0, d0 = C.c_longlong(), C.c_longlong()
            assert L.comdgb_transfer_bytes(a.s, C.byref(h0), C.byref(d0)) == 0
            ea = L.comdgb_nTimeSteps(3, a.s, 1e-15)
            h1, d1 = C.c_longlong(), C.c_longlong()
            assert L.comdgb_transfer_bytes(a.s, C.byref(h1), C.byref(d1)) == 0
        finally:
            L.comdgb_detach(a.s)
        nb, ntot = a.s.contents.nboxes, a.s.contents.ntot
        assert h1.value - h0.value == 4 * nb + 64 * ntot
        assert d1.value - d0.value == 4 * nb + 64 * ntot + 48 * ntot
        assert ea == eb
        assert slots_equal(a.s, b.s, ("id", "iType", "mass", "r", "p", "f", "rho", "fi"))
    finally:
        a.close()
        b.close()


@pytest.mark.gpu
def test_eager_call_after_host_array_moved(oracle):
    """The transfer kernels address the arrays registered at attach; when the
    caller moves one (here r to a new buffer) the call copies from the
    current pointers instead, with the same results as a device handle."""
    a = Case(oracle, cg.POT_EAM_CHEBY, n=(8, 8, 8), amp=0.05, temp=600.0)
    b = Case(oracle, cg.POT_EAM_CHEBY, n=(8, 8, 8), amp=0.05, temp=600.0)
    L = cg.load()
    try:
        o = cg.opts(cg.POT_EAM_CHEBY, cg.PREC_FP64, True, cheby_from_host=True,
                    per_step_lists=True)
        d = cg.DeviceSim(b.s, o)
        try:
            eb = d.steps(3, 1e-15)[0]
            d.download(b.s)
        finally:
            d.close()
        assert L.comdgb_attach(a.s, C.byref(o)) == 0
        # the address itself: a pointer field read from a ctypes structure
        # is a view of the field and would follow the reassignment
        orig = C.cast(a.s.contents.r, C.c_void_p).value
        moved = np.array(slot_views(a.s)["r"], copy=True)
        try:
            a.s.contents.r = moved.ctypes.data_as(C.POINTER(C.c_double))
            ea = L.comdgb_nTimeSteps(3, a.s, 1e-15)
        finally:
            a.s.contents.r = C.cast(orig, C.POINTER(C.c_double))
            L.comdgb_detach(a.s)
        assert C.cast(a.s.contents.r, C.c_void_p).value == orig
        slot_views(a.s)["r"][:] = moved
        assert ea == eb
        assert slots_equal(a.s, b.s, ("id", "iType", "mass", "r", "p", "f", "rho", "fi"))
    finally:
        a.close()
        b.close()
