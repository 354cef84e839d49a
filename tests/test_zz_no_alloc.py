"""The allocation-free binning entry point (comdgb_put_atoms_noalloc).

Callers that cannot allocate device memory while they run -- an engine that
owns all GPU memory in its own arena, latency-critical loops where
cudaMalloc's implicit synchronisation would stall the GPU -- bin atoms with
this entry point: they pass device buffers they already own, and the library
uses a fixed scratch array it holds for the life of the process.  This test (the caller here, which may
allocate) makes those buffers with the CUDA runtime, calls the entry point
twice in a row on two different inputs through the C ABI, and checks each
result against comdgb_put_atoms, exactly (binning is integer and exact FP64
work, compared exactly like the other binning tests).  The file is named so
that pytest collects it after every other test.  The error statuses
(box out of range, including a NaN coordinate, and a box of more than 64
atoms) are checked too, each followed by a valid call on a created stream
that must clear the status the failing call left in the shared array.
"""
import ctypes as C
import ctypes.util
import glob
import os

import numpy as np
import pytest

import comd_gb300 as cg
from comd_gb300.abi import occupied_mask, slot_views

pytestmark = pytest.mark.gpu


def _cudart():
    names = []
    found = ctypes.util.find_library("cudart")
    if found:
        names.append(found)
    for d in ("/usr/local/cuda/lib64", "/usr/local/cuda/targets/sbsa-linux/lib",
              "/usr/local/cuda/targets/x86_64-linux/lib"):
        names += sorted(glob.glob(os.path.join(d, "libcudart.so*")))
    for n in names:
        try:
            rt = C.CDLL(n)
        except OSError:
            continue
        rt.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
        rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
        rt.cudaFree.argtypes = [C.c_void_p]
        rt.cudaSetDevice.argtypes = [C.c_int]
        rt.cudaStreamCreate.argtypes = [C.POINTER(C.c_void_p)]
        rt.cudaStreamDestroy.argtypes = [C.c_void_p]
        rt.cudaStreamSynchronize.argtypes = [C.c_void_p]
        rt.cudaGetDevice.argtypes = [C.POINTER(C.c_int)]
        return rt
    pytest.skip("CUDA runtime library not found")


class DevBuf:
    def __init__(self, rt, nbytes):
        self.rt = rt
        self.ptr = C.c_void_p()
        assert rt.cudaMalloc(C.byref(self.ptr), max(int(nbytes), 8)) == 0
        self.nbytes = nbytes

    def put(self, arr):
        arr = np.ascontiguousarray(arr)
        assert arr.nbytes <= self.nbytes
        assert self.rt.cudaMemcpy(self.ptr, arr.ctypes.data, arr.nbytes, 1) == 0

    def get(self, dtype, shape):
        out = np.empty(shape, dtype)
        assert self.rt.cudaMemcpy(out.ctypes.data, self.ptr, out.nbytes, 2) == 0
        return out

    def free(self):
        self.rt.cudaFree(self.ptr)


def _inputs(s, seed):
    """atoms of a lattice in world coordinates, shuffled, some outside the box"""
    v = slot_views(s)
    occ = (np.arange(64)[None, :] < v["natoms"][:, None])
    boxes = np.nonzero(occ)[0]
    xyz = v["r"][occ.reshape(-1)] + v["dcenter"][boxes]
    rng = np.random.default_rng(seed)
    xyz = xyz + rng.normal(scale=0.3, size=xyz.shape)
    order = rng.permutation(len(xyz))
    xyz = np.ascontiguousarray(xyz[order])
    n = len(xyz)
    return (xyz, np.ascontiguousarray(rng.normal(size=(n, 3))),
            np.ascontiguousarray(rng.permutation(n).astype(np.int32)),
            np.ascontiguousarray(rng.integers(0, 3, n).astype(np.int32)),
            np.ascontiguousarray(rng.uniform(60, 70, n)))


def test_put_atoms_noalloc_matches_put_atoms_twice():
    L = cg.load()
    rt = _cudart()
    assert rt.cudaSetDevice(0) == 0
    pot = cg.eam_potential("cu")
    s = cg.fcc(10, 10, 10, 3.615, 1.0, 1.0, pot)  # 8 x 8 x 8 boxes
    nb = s.contents.nboxes
    ns = nb * 64
    assert nb <= 16384
    geo = ((C.c_int * 3)(*s.contents.nbx), (C.c_double * 3)(*s.contents.bounds),
           (C.c_double * 3)(*s.contents.boxsize))
    dcen = np.ascontiguousarray(slot_views(s)["dcenter"])
    n = s.contents.ntot
    bufs = {k: DevBuf(rt, sz) for k, sz in dict(
        dcenter=dcen.nbytes, xyz=n * 24, pxyz=n * 24, ids=n * 4, types=n * 4, masses=n * 8,
        natoms=nb * 4, id=ns * 4, itype=ns * 4, mass=ns * 8, r=ns * 24, p=ns * 24).items()}
    try:
        bufs["dcenter"].put(dcen)
        for call, seed in enumerate((11, 12)):  # two calls in a row, different inputs
            xyz, pxyz, ids, types, masses = _inputs(s, seed)
            # existing entry point on a host simulation with the same domains
            ref = cg.fcc(10, 10, 10, 3.615, 1.0, 1.0, pot)
            slot_views(ref)["natoms"][:] = 0
            ref.contents.ntot = 0
            assert L.comdgb_put_atoms(ref, n, xyz.ctypes.data, pxyz.ctypes.data, ids.ctypes.data,
                                      types.ctypes.data, masses.ctypes.data, 0) == 0
            for k, a in dict(xyz=xyz, pxyz=pxyz, ids=ids, types=types, masses=masses).items():
                bufs[k].put(a)
            rc = L.comdgb_put_atoms_noalloc(
                geo[0], geo[1], geo[2], bufs["dcenter"].ptr, n, bufs["xyz"].ptr,
                bufs["pxyz"].ptr, bufs["ids"].ptr, bufs["types"].ptr, bufs["masses"].ptr,
                bufs["natoms"].ptr, bufs["id"].ptr, bufs["itype"].ptr, bufs["mass"].ptr,
                bufs["r"].ptr, bufs["p"].ptr, 0, None)
            assert rc == 0, cg.lib.last_error()
            v = slot_views(ref)
            natoms = bufs["natoms"].get(np.int32, (nb,))
            assert np.array_equal(natoms, v["natoms"]), f"call {call}"
            m = occupied_mask(ref)
            got = dict(id=bufs["id"].get(np.int32, (ns,)), iType=bufs["itype"].get(np.int32, (ns,)),
                       mass=bufs["mass"].get(np.float64, (ns,)),
                       r=bufs["r"].get(np.float64, (ns, 3)), p=bufs["p"].get(np.float64, (ns, 3)))
            for k, a in got.items():
                assert np.array_equal(a[m], v[k][m]), f"call {call}: {k}"
            cg.free_host(ref)
    finally:
        for b in bufs.values():
            b.free()
        cg.free_host(s)


def test_put_atoms_noalloc_rejects_large_grids():
    L = cg.load()
    nbx = (C.c_int * 3)(64, 64, 8)  # 32768 boxes > 16384
    bounds = (C.c_double * 3)(100.0, 100.0, 100.0)
    bs = (C.c_double * 3)(100 / 64, 100 / 64, 12.5)
    dummy = C.c_void_p(1)
    rc = L.comdgb_put_atoms_noalloc(nbx, bounds, bs, dummy, 0, None, None, None, None, None,
                                    dummy, dummy, dummy, dummy, dummy, dummy, 0, None)
    assert rc == -1  # COMDGB_ERR_ARG
    assert "allocation-free limit" in cg.lib.last_error()


def _bin_case(s, seed):
    """geometry, device buffers and the reference result (comdgb_put_atoms)
    of one seeded input on the domains of host simulation s"""
    L = cg.load()
    pot = cg.eam_potential("cu")
    xyz, pxyz, ids, types, masses = _inputs(s, seed)
    n = len(xyz)
    ref = cg.fcc(10, 10, 10, 3.615, 1.0, 1.0, pot)
    slot_views(ref)["natoms"][:] = 0
    ref.contents.ntot = 0
    assert L.comdgb_put_atoms(ref, n, xyz.ctypes.data, pxyz.ctypes.data, ids.ctypes.data,
                              types.ctypes.data, masses.ctypes.data, 0) == 0
    return (xyz, pxyz, ids, types, masses), ref


def test_put_atoms_noalloc_error_statuses_then_valid_call():
    """-12 (an atom two periods outside, and a NaN coordinate) and -11 (65
    atoms in one box); each failing call is followed by a valid call on a
    non-default stream that returns 0 and matches comdgb_put_atoms, and the
    caller's current device is the same after every call"""
    L = cg.load()
    rt = _cudart()
    assert rt.cudaSetDevice(0) == 0
    pot = cg.eam_potential("cu")
    s = cg.fcc(10, 10, 10, 3.615, 1.0, 1.0, pot)
    nb = s.contents.nboxes
    ns = nb * 64
    geo = ((C.c_int * 3)(*s.contents.nbx), (C.c_double * 3)(*s.contents.bounds),
           (C.c_double * 3)(*s.contents.boxsize))
    dcen = np.ascontiguousarray(slot_views(s)["dcenter"])
    n = s.contents.ntot
    bufs = {k: DevBuf(rt, sz) for k, sz in dict(
        dcenter=dcen.nbytes, xyz=n * 24, pxyz=n * 24, ids=n * 4, types=n * 4, masses=n * 8,
        natoms=nb * 4, id=ns * 4, itype=ns * 4, mass=ns * 8, r=ns * 24, p=ns * 24).items()}
    stream = C.c_void_p()
    assert rt.cudaStreamCreate(C.byref(stream)) == 0

    def call(arrays, nn, st):
        for k, a in zip(("xyz", "pxyz", "ids", "types", "masses"), arrays):
            bufs[k].put(a)
        return L.comdgb_put_atoms_noalloc(
            geo[0], geo[1], geo[2], bufs["dcenter"].ptr, nn, bufs["xyz"].ptr, bufs["pxyz"].ptr,
            bufs["ids"].ptr, bufs["types"].ptr, bufs["masses"].ptr, bufs["natoms"].ptr,
            bufs["id"].ptr, bufs["itype"].ptr, bufs["mass"].ptr, bufs["r"].ptr, bufs["p"].ptr, 0,
            st)

    def current_device():
        d = C.c_int(-1)
        assert rt.cudaGetDevice(C.byref(d)) == 0
        return d.value

    try:
        bufs["dcenter"].put(dcen)
        L0 = np.array(s.contents.bounds[:3])
        good, ref = _bin_case(s, 21)
        far = [a.copy() for a in good]
        far[0][5] = far[0][5] + 2.0 * L0  # two periods outside: not wrapped into the grid
        nan = [a.copy() for a in good]
        nan[0][7, 1] = np.nan
        crowd = [a.copy() for a in good]
        crowd[0][:65] = np.array(slot_views(s)["dcenter"][3]) + 0.5  # 65 atoms in box 3
        for bad, code in ((far, -12), (nan, -12), (crowd, -11)):
            rc = call(bad, n, None)
            assert rc == code, (code, rc, cg.lib.last_error())
            assert current_device() == 0
            rc = call(good, n, stream)
            assert rc == 0, cg.lib.last_error()
            assert rt.cudaStreamSynchronize(stream) == 0
            assert current_device() == 0
            v = slot_views(ref)
            assert np.array_equal(bufs["natoms"].get(np.int32, (nb,)), v["natoms"])
            m = occupied_mask(ref)
            got = dict(id=bufs["id"].get(np.int32, (ns,)),
                       iType=bufs["itype"].get(np.int32, (ns,)),
                       mass=bufs["mass"].get(np.float64, (ns,)),
                       r=bufs["r"].get(np.float64, (ns, 3)), p=bufs["p"].get(np.float64, (ns, 3)))
            for k, a in got.items():
                assert np.array_equal(a[m], v[k][m]), f"after {code}: {k}"
        cg.free_host(ref)
    finally:
        rt.cudaStreamDestroy(stream)
        for b in bufs.values():
            b.free()
        cg.free_host(s)
