"""ctypes mirror of include/comdgb_simflat.h (the reference's -DDOUBLE data model).

The structs match CoMD src-flat member for member:
``simflat_t`` src-flat/include/pmdTypes.h:104-141, ``potentialarray_t``
src-flat/include/eamTypes.h:68-74, ``eampotential_t`` eamTypes.h:92-101,
``eam_cheby_t`` eamTypes.h:104-114, ``ljpotential_t`` src-flat/include/ljTypes.h:72-81.
``slot_views`` exposes a simulation's per-slot arrays as numpy views so
tests can read and write them without copies.
"""
import ctypes as C

import numpy as np

MAXATOMS = 64
NUMNEIGHBORS = 27

FORCE_FN = C.CFUNCTYPE(C.c_int, C.c_void_p)
DESTROY_FN = C.CFUNCTYPE(None, C.c_void_p)


class PotentialArray(C.Structure):
    _fields_ = [("n", C.c_int), ("x0", C.c_double), ("xn", C.c_double),
                ("invDx", C.c_double), ("values", C.POINTER(C.c_double))]


class BasePotential(C.Structure):
    _fields_ = [("cutoff", C.c_double), ("mass", C.c_double),
                ("force", C.c_void_p), ("destroy", C.c_void_p)]


class EamPotential(C.Structure):
    _fields_ = [("cutoff", C.c_double), ("mass", C.c_double),
                ("force", C.c_void_p), ("destroy", C.c_void_p),
                ("phi", C.POINTER(PotentialArray)), ("rho", C.POINTER(PotentialArray)),
                ("f", C.POINTER(PotentialArray)), ("lat", C.c_double)]


class EamCheby(C.Structure):
    _fields_ = [("cutoff", C.c_double), ("mass", C.c_double),
                ("phi", C.POINTER(PotentialArray)), ("rho", C.POINTER(PotentialArray)),
                ("f", C.POINTER(PotentialArray)), ("dphi", C.POINTER(PotentialArray)),
                ("drho", C.POINTER(PotentialArray)), ("df", C.POINTER(PotentialArray)),
                ("lat", C.c_double)]


class LjPotential(C.Structure):
    _fields_ = [("cutoff", C.c_double), ("mass", C.c_double),
                ("force", C.c_void_p), ("destroy", C.c_void_p),
                ("sigma", C.c_double), ("epsilon", C.c_double)]


class SimFlat(C.Structure):
    _fields_ = [("stateflag", C.c_int), ("nbx", C.c_int * 3), ("nboxes", C.c_int),
                ("ntot", C.c_int), ("bounds", C.c_double * 3), ("boxsize", C.c_double * 3),
                ("dcenter", C.POINTER(C.c_double)), ("natoms", C.POINTER(C.c_int)),
                ("id", C.POINTER(C.c_int)), ("iType", C.POINTER(C.c_int)),
                ("mass", C.POINTER(C.c_double)), ("r", C.POINTER(C.c_double)),
                ("p", C.POINTER(C.c_double)), ("f", C.POINTER(C.c_double)),
                ("rho", C.POINTER(C.c_double)), ("fi", C.POINTER(C.c_double)),
                ("e", C.c_double), ("nAtoms", C.c_int),
                ("pot", C.POINTER(BasePotential)), ("comment", C.c_char_p),
                ("stress", C.c_double), ("defgrad", C.c_double), ("bf", C.c_double),
                ("ch_pot", C.POINTER(EamCheby))]


def _view(ptr, shape, dtype):
    n = int(np.prod(shape))
    if n == 0:
        return np.zeros(shape, dtype)
    ctype = C.c_double if dtype == np.float64 else C.c_int
    buf = C.cast(ptr, C.POINTER(ctype * n)).contents
    return np.frombuffer(buf, dtype=dtype).reshape(shape)


def slot_views(sp):
    """numpy views (no copy) over the per-slot arrays of a SimFlat pointer."""
    s = sp.contents
    nb = s.nboxes
    ns = nb * MAXATOMS
    return {
        "natoms": _view(s.natoms, (nb,), np.int32),
        "dcenter": _view(s.dcenter, (nb, 3), np.float64),
        "id": _view(s.id, (ns,), np.int32),
        "iType": _view(s.iType, (ns,), np.int32),
        "mass": _view(s.mass, (ns,), np.float64),
        "r": _view(s.r, (ns, 3), np.float64),
        "p": _view(s.p, (ns, 3), np.float64),
        "f": _view(s.f, (ns, 4), np.float64),
        "rho": _view(s.rho, (ns,), np.float64),
        "fi": _view(s.fi, (ns,), np.float64),
    }


def occupied_mask(sp):
    """boolean mask over slots: True where k < natoms[box]."""
    v = slot_views(sp)
    k = np.arange(MAXATOMS)[None, :]
    return (k < v["natoms"][:, None]).reshape(-1)


def by_id(sp, name):
    """per-atom array ``name`` reordered by atom id (occupied slots only)."""
    v = slot_views(sp)
    m = occupied_mask(sp)
    ids = v["id"][m]
    vals = v[name][m]
    out = np.empty_like(vals)
    out[ids] = vals
    return out
