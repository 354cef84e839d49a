"""TEST INFRASTRUCTURE ONLY: ctypes bindings of the CPU oracle and of the
reference compiled from its sources (oracle/_ref).

``Oracle`` wraps liboracle.so (the restatement in comd_oracle.c).
``RefLib`` wraps oracle/_ref/libcomdref_{table,cheby}.so when they exist
(they are built only where the reference sources are present).
"""
import ctypes as C

import numpy as np
import os
import subprocess
import threading

from comd_gb300.abi import EamCheby, EamPotential, LjPotential, SimFlat

HERE = os.path.dirname(os.path.abspath(__file__))
KIND_EAM_TABLE, KIND_EAM_CHEBY, KIND_LJ = 0, 1, 2
P_SIM = C.POINTER(SimFlat)

_lock = threading.Lock()
_oracle = None
_refs = {}


def reference_dir():
    """the reference source tree: $COMDGB_REFERENCE_DIR, else the directory
    `reference` beside the repository (None when neither holds src-flat)"""
    for d in (os.environ.get("COMDGB_REFERENCE_DIR"),
              os.path.join(os.path.dirname(HERE), os.pardir, "reference")):
        if d and os.path.exists(os.path.join(d, "src-flat", "eam.c")):
            return os.path.abspath(d)
    return None


def build(with_ref=True):
    """make the oracle (and oracle/_ref when the reference is present)."""
    target = "all" if with_ref else os.path.join(HERE, "liboracle.so")
    cmd = ["make", "-s", "-C", HERE, target]
    ref = reference_dir() if with_ref else None
    if ref:
        cmd.append("REF=" + ref)
    subprocess.run(cmd, check=True)


def _bind(lib):
    f = lib
    f.orc_set_periodic.argtypes = [C.c_int]
    f.orc_eam_read.restype = C.POINTER(EamPotential)
    f.orc_eam_read.argtypes = [C.c_char_p, C.c_char_p]
    f.orc_eam_free.argtypes = [C.c_void_p]
    f.orc_cheb_make.restype = C.POINTER(EamCheby)
    f.orc_cheb_make.argtypes = [C.c_void_p, C.c_int]
    f.orc_cheb_free.argtypes = [C.c_void_p]
    f.orc_cheb_eval.restype = C.c_double
    f.orc_cheb_eval.argtypes = [C.c_void_p, C.c_double]
    f.orc_table_eval.argtypes = [C.c_void_p, C.c_double, C.POINTER(C.c_double),
                                 C.POINTER(C.c_double)]
    f.orc_fcc.restype = P_SIM
    f.orc_fcc.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                          C.c_void_p, C.POINTER(C.c_int)]
    f.orc_sim_clone.restype = P_SIM
    f.orc_sim_clone.argtypes = [P_SIM]
    f.orc_sim_free.argtypes = [P_SIM]
    f.orc_alloc_domains.argtypes = [P_SIM]
    f.orc_put_atom.argtypes = [P_SIM, C.c_int, C.c_int, C.c_double] + [C.c_double] * 6
    f.orc_rebox_all.argtypes = [P_SIM]
    f.orc_neighbor_boxes.argtypes = [P_SIM, C.c_int, C.POINTER(C.c_int)]
    f.orc_eam_force.argtypes = [P_SIM, C.c_int]
    f.orc_lj_force.argtypes = [P_SIM]
    f.orc_force.argtypes = [P_SIM, C.c_int]
    f.orc_ntimesteps.argtypes = [C.c_int, P_SIM, C.c_double, C.c_int]
    f.orc_advance_velocity.argtypes = [P_SIM, C.c_double]
    f.orc_advance_positions.argtypes = [P_SIM, C.c_double]
    f.orc_seed_apply.argtypes = [P_SIM, C.c_uint64, C.c_int, C.c_double, C.c_double,
                                 C.c_double]
    f.orc_kinetic.restype = C.c_double
    f.orc_kinetic.argtypes = [P_SIM]
    f.orc_lj_make.restype = C.POINTER(LjPotential)
    f.orc_lj_make.argtypes = [C.c_double] * 4
    f.orc_free.argtypes = [C.c_void_p]
    f.orc_read_clsman.restype = P_SIM
    f.orc_read_clsman.argtypes = [C.c_char_p, C.c_void_p, C.c_double, C.POINTER(C.c_int)]
    D = C.POINTER(C.c_double)
    f.orc_virial.argtypes = [P_SIM, C.c_int, D, D, D]
    f.orc_strained.restype = P_SIM
    f.orc_strained.argtypes = [P_SIM, D]
    f.orc_centro.argtypes = [P_SIM, C.c_int, D, D, D]
    f.orc_cheb_set.argtypes = [C.c_void_p, D, D, D]
    f.orc_eam_cheb_grad.argtypes = [P_SIM, D, D, D, D, D]
    f.orc_lj_grad.argtypes = [P_SIM, D, D, D, D, D]
    return lib


def oracle_lib():
    global _oracle
    with _lock:
        if _oracle is None:
            path = os.path.join(HERE, "liboracle.so")
            if not os.path.exists(path):
                build(with_ref=False)
            _oracle = _bind(C.CDLL(path))
        return _oracle


class Oracle:
    """Thin OO helper over liboracle.so (all state is in C structs)."""

    def __init__(self):
        self.lib = oracle_lib()

    def eam(self, potdir, name="cu"):
        p = self.lib.orc_eam_read(potdir.encode(), name.encode())
        if not p:
            raise IOError(f"cannot read EAM potential {name} from {potdir}")
        return p

    def cheby(self, pot, n=32):
        return self.lib.orc_cheb_make(pot, n)

    def read_clsman(self, path, pot, bf=1.0):
        """fromFileGzip's arithmetic on an uncompressed clsman file"""
        st = C.c_int(0)
        s = self.lib.orc_read_clsman(path.encode(), C.cast(pot, C.c_void_p), bf, C.byref(st))
        if not s:
            raise IOError(f"oracle clsman read failed: {st.value}")
        return s

    def cheb_set(self, ch, coef, x0, xn):
        """replace the base series (phi, rho, F) and derive the derivative series"""
        P = C.POINTER(C.c_double)
        c = np.ascontiguousarray(coef, dtype=np.float64)
        a = np.ascontiguousarray(x0, dtype=np.float64)
        b = np.ascontiguousarray(xn, dtype=np.float64)
        self.lib.orc_cheb_set(ch, c.ctypes.data_as(P), a.ctypes.data_as(P), b.ctypes.data_as(P))

    def grad(self, s, kind, target=None):
        """(U, dU/dp, L, dL/dp) for EAM Chebyshev (96 parameters) or LJ (2)"""
        P = C.POINTER(C.c_double)
        n = 2 if kind == "lj" else 96
        gu, gl = np.zeros(n), np.zeros(n)
        e, loss = C.c_double(), C.c_double()
        t = None if target is None else np.ascontiguousarray(target, dtype=np.float64)
        tp = t.ctypes.data_as(P) if t is not None else None
        fn = self.lib.orc_lj_grad if kind == "lj" else self.lib.orc_eam_cheb_grad
        rc = fn(s, tp, C.byref(e), gu.ctypes.data_as(P), C.byref(loss),
                gl.ctypes.data_as(P) if t is not None else None)
        if rc:
            raise RuntimeError(f"oracle gradient failed: {rc}")
        return e.value, gu, loss.value, gl

    def virial(self, s, kind, atoms=False):
        """(W[6], K[6], per-slot stress [nslots, 6] or None) of the state after
        a force call; Voigt order xx yy zz yz xz xy"""
        P = C.POINTER(C.c_double)
        w, k = np.zeros(6), np.zeros(6)
        a = np.zeros((s.contents.nboxes * 64, 6)) if atoms else None
        rc = self.lib.orc_virial(s, kind, w.ctypes.data_as(P), k.ctypes.data_as(P),
                                 a.ctypes.data_as(P) if atoms else None)
        if rc:
            raise RuntimeError(f"oracle virial failed: {rc}")
        return w, k, a

    def centro(self, s, approx=False):
        """(per-slot centrosymmetry [nslots], min, max)"""
        P = C.POINTER(C.c_double)
        out = np.zeros(s.contents.nboxes * 64)
        lo, hi = C.c_double(), C.c_double()
        self.lib.orc_centro(s, int(approx), out.ctypes.data_as(P), C.byref(lo), C.byref(hi))
        return out, lo.value, hi.value

    def strained(self, s, scale):
        """copy of s under x_a -> scale[a] x_a (bounds and positions)"""
        sc = np.ascontiguousarray(scale, dtype=np.float64)
        t = self.lib.orc_strained(s, sc.ctypes.data_as(C.POINTER(C.c_double)))
        if not t:
            raise RuntimeError("oracle strained copy failed")
        return t

    def lj(self, sigma, epsilon, cutoff, mass):
        return self.lib.orc_lj_make(sigma, epsilon, cutoff, mass)

    def fcc(self, nx, ny, nz, lat, defgrad, bf, pot):
        st = C.c_int(0)
        s = self.lib.orc_fcc(nx, ny, nz, lat, defgrad, bf, C.cast(pot, C.c_void_p),
                             C.byref(st))
        if not s:
            raise RuntimeError(f"orc_fcc failed with code {st.value}")
        return s

    def clone(self, s):
        return self.lib.orc_sim_clone(s)

    def free(self, s):
        self.lib.orc_sim_free(s)

    def rebox(self, s):
        return self.lib.orc_rebox_all(s)

    def force(self, s, kind):
        return self.lib.orc_force(s, kind)

    def steps(self, s, n, dt, kind):
        return self.lib.orc_ntimesteps(n, s, dt, kind)

    def seed(self, s, seed, kind, amp, temp_k, mass_amu):
        self.lib.orc_seed_apply(s, seed, kind, amp, temp_k, mass_amu)

    def set_periodic(self, p):
        self.lib.orc_set_periodic(int(p))


class RefLib:
    """The reference src-flat compiled from its sources (FP64)."""

    def __init__(self, cheby=False):
        name = "libcomdref_cheby.so" if cheby else "libcomdref_table.so"
        path = os.path.join(HERE, "_ref", name)
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        lib = C.CDLL(path)
        lib.refh_eam_load.restype = C.c_void_p
        lib.refh_eam_load.argtypes = [C.c_char_p, C.c_char_p]
        lib.refh_lj_make.restype = C.c_void_p
        lib.refh_lj_make.argtypes = [C.c_double] * 4
        lib.refh_fcc.restype = P_SIM
        lib.refh_fcc.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                 C.c_double, C.c_void_p, C.c_int]
        lib.refh_seed_apply.argtypes = [P_SIM, C.c_uint64, C.c_int, C.c_double, C.c_double,
                                        C.c_double]
        lib.refh_rebox.argtypes = [P_SIM]
        lib.refh_force.argtypes = [P_SIM]
        lib.refh_ntimesteps.restype = C.c_double
        lib.refh_ntimesteps.argtypes = [C.c_int, P_SIM, C.c_double]
        lib.refh_set_periodic.argtypes = [C.c_int]
        lib.refh_read_clsman.restype = P_SIM
        lib.refh_write_clsman.argtypes = [P_SIM, C.c_char_p]
        lib.refh_read_tim.restype = P_SIM
        lib.refh_read_tim.argtypes = [C.c_char_p, C.c_double, C.c_void_p]
        lib.refh_set_comment.argtypes = [P_SIM, C.c_char_p]
        lib.refh_gz_ascii_write.argtypes = [P_SIM, C.c_char_p]
        lib.refh_print_it.argtypes = [P_SIM, C.c_char_p]
        lib.refh_read_clsman.argtypes = [C.c_char_p, C.c_double, C.c_void_p, C.c_int]
        self.lib = lib
        self.cheby = cheby


class RefCentro:
    """The reference visualiser's computeCentrosymmetry, compiled from its
    text by oracle/Makefile (exact, or the -DAPPROX_CENTROSYM greedy
    pairing), over a simulation's slot arrays."""

    def __init__(self, approx=False):
        name = "libcomdref_centro_approx.so" if approx else "libcomdref_centro.so"
        path = os.path.join(HERE, "_ref", name)
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        lib = C.CDLL(path)
        D = C.POINTER(C.c_double)
        lib.refc_centro.restype = C.c_int
        lib.refc_centro.argtypes = [C.c_int, C.POINTER(C.c_int), D, D, C.POINTER(C.c_int), D, D,
                                    C.POINTER(C.c_float)]
        self.lib = lib

    def centro(self, s):
        """(per-slot centrosymmetry [nslots], minCentro, maxCentro as floats)"""
        v = s.contents
        nb = v.nboxes
        nbx = (C.c_int * 3)(*v.nbx)
        bounds = (C.c_double * 3)(*v.bounds)
        out = np.zeros(nb * 64)
        mm = (C.c_float * 2)()
        D = C.POINTER(C.c_double)
        stride = self.lib.refc_centro(nb, nbx, bounds, C.cast(v.dcenter, D), v.natoms,
                                      C.cast(v.r, D), out.ctypes.data_as(D), mm)
        if stride != 64:
            raise RuntimeError(f"reference MAXATOMS {stride} != 64")
        return out, mm[0], mm[1]


_centro_refs = {}


def ref_centro(approx=False):
    """RefCentro or None when oracle/_ref holds no centrosymmetry build."""
    key = bool(approx)
    with _lock:
        if key not in _centro_refs:
            try:
                _centro_refs[key] = RefCentro(approx)
            except (FileNotFoundError, OSError):
                _centro_refs[key] = None
        return _centro_refs[key]


def ref_lib(cheby=False):
    """RefLib or None when oracle/_ref was not built on this machine."""
    key = bool(cheby)
    with _lock:
        if key not in _refs:
            try:
                _refs[key] = RefLib(cheby)
            except (FileNotFoundError, OSError):
                _refs[key] = None
        return _refs[key]
