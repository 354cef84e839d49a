"""ctypes bindings of libcomdgb.so (the C ABI declared in include/comdgb.h).

Python only calls the library here: every computation runs in the library's
CUDA kernels.  Loading fails loudly if the library is missing; there is no
CPU fallback.
"""
import ctypes as C
import os
import threading

import numpy as np

from .abi import EamCheby, EamPotential, LjPotential, SimFlat

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcomdgb.so")
POT_DIR = os.path.join(HERE, "pots")

POT_EAM_TABLE, POT_EAM_CHEBY, POT_LJ = 0, 1, 2
CLSMAN_BINARY, CLSMAN_TEXT_GZ, CLSMAN_TEXT = 0, 1, 2
PREC_FP64, PREC_MIXED = 0, 1
DISP_NONE, DISP_UNIFORM, DISP_GAUSSIAN = 0, 1, 2
ERR_MAXATOMS, ERR_BOXRANGE, ERR_NOBOX = -11, -12, -3

# s -> t0 (src-flat/include/constants.h:61), amu -> m_e, k_B in Ha/K, eV in Ha
BOHR_PER_ATU = 0.529 / 2.418e-17
AMU_TO_ME = 1822.83
KB_HA = 3.166811563e-6
EV_TO_HA = 1.0 / 27.211386245988

P_SIM = C.POINTER(SimFlat)


class Opts(C.Structure):
    _fields_ = [("potential", C.c_int), ("precision", C.c_int), ("periodic", C.c_int),
                ("device", C.c_int), ("n_cheby", C.c_int), ("cheby_from_host", C.c_int),
                ("list_mode", C.c_int), ("skin", C.c_double)]


class Tune(C.Structure):
    _fields_ = [("box_factor", C.c_double), ("skin", C.c_double), ("build_threads", C.c_int),
                ("build_atoms", C.c_int), ("pass2_threads", C.c_int),
                ("ms_per_step", C.c_double), ("from_cache", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class ComdgbError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"libcomdgb error {code}: {msg}")
        self.code = code


_lock = threading.Lock()
_lib = None


def _bind(lib):
    L = lib
    L.comdgb_default_opts.argtypes = [C.POINTER(Opts)]
    L.comdgb_last_error.argtypes = [C.c_char_p, C.c_int]
    L.comdgb_version.restype = C.c_char_p
    L.comdgb_attach.argtypes = [P_SIM, C.POINTER(Opts)]
    L.comdgb_force.argtypes = [C.c_void_p]
    L.comdgb_nTimeSteps.restype = C.c_double
    L.comdgb_nTimeSteps.argtypes = [C.c_int, P_SIM, C.c_double]
    L.comdgb_reBoxAll.argtypes = [P_SIM]
    L.comdgb_detach.argtypes = [P_SIM]
    L.comdgb_sim_create.argtypes = [P_SIM, C.POINTER(Opts), C.POINTER(C.c_void_p)]
    L.comdgb_sim_destroy.argtypes = [C.c_void_p]
    L.comdgb_sim_upload.argtypes = [C.c_void_p, P_SIM]
    L.comdgb_sim_download.argtypes = [C.c_void_p, P_SIM]
    L.comdgb_sim_force.argtypes = [C.c_void_p]
    L.comdgb_sim_steps.argtypes = [C.c_void_p, C.c_int, C.c_double]
    L.comdgb_sim_rebox.argtypes = [C.c_void_p]
    L.comdgb_sim_advance_velocity.argtypes = [C.c_void_p, C.c_double]
    L.comdgb_sim_advance_positions.argtypes = [C.c_void_p, C.c_double]
    L.comdgb_sim_energy.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.comdgb_sim_kinetic.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
    L.comdgb_sim_pair_count.argtypes = [C.c_void_p, C.POINTER(C.c_longlong)]
    L.comdgb_sim_synchronize.argtypes = [C.c_void_p]
    L.comdgb_sim_timed_steps.argtypes = [C.c_void_p, C.c_int, C.c_double,
                                         C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int]
    L.comdgb_sim_graph_kernels.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.comdgb_sim_step_launches.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_longlong)]
    L.comdgb_sim_rebuild_launches.argtypes = [C.c_void_p, C.POINTER(C.c_int)]
    L.comdgb_fp32_fma_peak.argtypes = [C.c_int, C.POINTER(C.c_double)]
    L.comdgb_round_f32.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_float), C.c_long]
    D = C.POINTER(C.c_double)
    L.comdgb_sim_set_cheby.argtypes = [C.c_void_p, D, D, D]
    L.comdgb_sim_get_cheby.argtypes = [C.c_void_p, D, D, D]
    L.comdgb_sim_set_lj.argtypes = [C.c_void_p, C.c_double, C.c_double]
    L.comdgb_sim_energy_grad.argtypes = [C.c_void_p, D, D]
    L.comdgb_sim_force_loss_grad.argtypes = [C.c_void_p, D, D, D]
    L.comdgb_sim_traj_energy_grad.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_int, D, D]
    L.comdgb_sim_graph_steps.argtypes = [C.c_void_p, C.c_int, C.c_double,
                                         C.POINTER(C.c_float)]
    L.comdgb_batch_create.argtypes = [C.POINTER(P_SIM), C.c_int, C.c_void_p,
                                      C.POINTER(C.c_void_p)]
    L.comdgb_batch_replicas.argtypes = [C.c_void_p]
    L.comdgb_batch_upload.argtypes = [C.c_void_p, C.c_int, P_SIM]
    L.comdgb_batch_download.argtypes = [C.c_void_p, C.c_int, P_SIM]
    L.comdgb_batch_energies.argtypes = [C.c_void_p, D, D]
    L.comdgb_sim_virial.argtypes = [C.c_void_p, D, D, D]
    L.comdgb_sim_gather.argtypes = [C.c_void_p, C.c_int, D]
    L.comdgb_read_tim.restype = P_SIM
    L.comdgb_read_tim.argtypes = [C.c_char_p, C.c_void_p, C.c_double, D, C.c_int,
                                  C.POINTER(C.c_int)]
    L.comdgb_sim_centrosymmetry.argtypes = [C.c_void_p, C.c_int, C.c_int, D, D, D]
    L.comdgb_sim_write_clsman.argtypes = [C.c_void_p, C.c_int, C.c_char_p, C.c_int, C.c_char_p]
    L.comdgb_writeClsman.argtypes = [P_SIM, C.c_char_p]
    L.comdgb_gzASCIIWrite.argtypes = [P_SIM, C.c_char_p]
    L.comdgb_printIt.argtypes = [P_SIM, C.c_void_p]
    L.comdgb_batch_virial.argtypes = [C.c_void_p, C.c_int, D, D, D]
    L.comdgb_sim_atom_stress.argtypes = [C.c_void_p, C.c_int, D]
    L.comdgb_sim_set_launch.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int]
    L.comdgb_sim_set_merge_rebox.argtypes = [C.c_void_p, C.c_int]
    L.comdgb_sim_set_list_capacity.argtypes = [C.c_void_p, C.c_int]
    L.comdgb_batch_autotune.argtypes = [C.POINTER(P_SIM), C.c_int, C.c_void_p,
                                        C.POINTER(C.c_double), C.c_int,
                                        C.POINTER(C.c_double), C.c_int, C.c_int, C.c_double,
                                        C.c_char_p, C.POINTER(Tune)]
    L.comdgb_sim_apply_tune.argtypes = [C.c_void_p, C.POINTER(Tune)]
    L.comdgb_graph_node_cost.argtypes = [C.c_int, C.POINTER(C.c_double)]
    L.comdgb_grid_barrier_cost.argtypes = [C.c_int, C.POINTER(C.c_double)]
    L.comdgb_rebin_host.restype = P_SIM
    L.comdgb_rebin_host.argtypes = [P_SIM, C.c_double, C.POINTER(C.c_int)]
    L.comdgb_sim_set_pair_table.argtypes = [C.c_void_p, C.c_int]
    L.comdgb_set_lazy.argtypes = [P_SIM, C.c_int]
    L.comdgb_sync_to_host.argtypes = [P_SIM]
    L.comdgb_sync_to_device.argtypes = [P_SIM]
    L.comdgb_transfer_bytes.argtypes = [P_SIM, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]
    L.comdgb_sim_list_info.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                       C.POINTER(C.c_longlong)]
    L.comdgb_kernel_name.restype = C.c_char_p
    L.comdgb_kernel_name.argtypes = [C.c_void_p, C.c_int]
    L.comdgb_eam_read.restype = C.POINTER(EamPotential)
    L.comdgb_eam_read.argtypes = [C.c_char_p, C.c_char_p]
    L.comdgb_eam_free.argtypes = [C.c_void_p]
    L.comdgb_cheb_make.restype = C.POINTER(EamCheby)
    L.comdgb_cheb_make.argtypes = [C.c_void_p, C.c_int, C.c_int]
    L.comdgb_cheb_free.argtypes = [C.c_void_p]
    L.comdgb_lj_make.restype = C.POINTER(LjPotential)
    L.comdgb_lj_make.argtypes = [C.c_double] * 4
    L.comdgb_lj_free.argtypes = [C.c_void_p]
    L.comdgb_read_clsman.restype = P_SIM
    L.comdgb_read_clsman.argtypes = [C.c_char_p, C.c_void_p, C.c_double, C.c_int,
                                     C.POINTER(C.c_int)]
    L.comdgb_fcc.restype = P_SIM
    L.comdgb_fcc.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                             C.c_void_p, C.POINTER(C.c_int)]
    L.comdgb_seed.argtypes = [P_SIM, C.c_uint64, C.c_int, C.c_double, C.c_double, C.c_double]
    L.comdgb_sim_free_host.argtypes = [P_SIM]
    L.comdgb_rebox_host.argtypes = [P_SIM, C.c_int, C.c_int]
    L.comdgb_put_atoms.argtypes = [P_SIM, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.c_void_p, C.c_int]
    L.comdgb_put_atoms_noalloc.argtypes = (
        [C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_void_p, C.c_int]
        + [C.c_void_p] * 5 + [C.c_void_p] * 6 + [C.c_int, C.c_void_p])
    return lib


def load(build_if_missing=True):
    """The loaded libcomdgb.so (built in-tree on first use if absent)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH) and build_if_missing:
                from .build import build
                build()
            if not os.path.exists(LIB_PATH):
                raise ImportError(f"libcomdgb.so not built at {LIB_PATH}")
            _lib = _bind(C.CDLL(LIB_PATH))
        return _lib


def fp32_peak_tflops(device=0):
    v = C.c_double()
    check(load().comdgb_fp32_fma_peak(device, C.byref(v)))
    return v.value


def round_f32(x):
    """FP64 -> FP32 (nearest, ties to even) by the library's integer routine."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty(x.shape, dtype=np.float32)
    check(load().comdgb_round_f32(x.ctypes.data_as(C.POINTER(C.c_double)),
                                  y.ctypes.data_as(C.POINTER(C.c_float)), x.size))
    return y


def last_error():
    buf = C.create_string_buffer(512)
    load().comdgb_last_error(buf, 512)
    return buf.value.decode(errors="replace")


def check(rc):
    if rc < 0:
        raise ComdgbError(rc, last_error())
    return rc


def opts(potential=POT_EAM_TABLE, precision=PREC_FP64, periodic=True, device=0,
         cheby_from_host=False, per_step_lists=False, skin=None):
    o = Opts()
    load().comdgb_default_opts(C.byref(o))
    o.list_mode = 1 if per_step_lists else 0
    if skin is not None:
        o.skin = skin
    o.potential = potential
    o.precision = precision
    o.periodic = int(periodic)
    o.device = device
    o.cheby_from_host = int(cheby_from_host)
    return o


class Potential:
    """Owns a host potential struct made by the library."""

    def __init__(self, ptr, kind, free_fn):
        self.ptr = ptr
        self.kind = kind
        self._free = free_fn

    @property
    def base(self):
        return C.cast(self.ptr, C.c_void_p)

    def close(self):
        if self.ptr:
            self._free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def eam_potential(name="cu", potdir=POT_DIR):
    L = load()
    p = L.comdgb_eam_read(potdir.encode(), name.encode())
    if not p:
        raise IOError(f"cannot read EAM potential {name} from {potdir}")
    return Potential(p, "eam", L.comdgb_eam_free)


def lj_potential(sigma, epsilon, cutoff, mass):
    L = load()
    return Potential(L.comdgb_lj_make(sigma, epsilon, cutoff, mass), "lj", L.comdgb_lj_free)


DATA_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")


def read_clsman(path, pot, bf=1.0, device=0):
    """comdgb_read_clsman: a clsman file into a new host simflat_t (atoms
    binned on the GPU `device`, or on the host for device < 0)"""
    L = load()
    st = C.c_int(0)
    s = L.comdgb_read_clsman(path.encode(), pot.base, bf, device, C.byref(st))
    if not s:
        raise ComdgbError(st.value, "comdgb_read_clsman failed: " + last_error())
    return s


def read_tim(path, pot, bf=1.0, bounds=None, device=0):
    """comdgb_read_tim: a FileAtom file into a new host simflat_t (the
    reference's fixed bounds unless `bounds` is given)"""
    L = load()
    st = C.c_int(0)
    b = None if bounds is None else (C.c_double * 3)(*bounds)
    s = L.comdgb_read_tim(path.encode(), pot.base, bf, b, device, C.byref(st))
    if not s:
        raise ComdgbError(st.value, "comdgb_read_tim failed: " + last_error())
    return s


def write_clsman_host(s, path, binary=True):
    """the drop-ins comdgb_writeClsman / comdgb_gzASCIIWrite on a host
    simflat_t (gathered on the device when it is attached, else on the host)"""
    L = load()
    fn = L.comdgb_writeClsman if binary else L.comdgb_gzASCIIWrite
    check(fn(s, path.encode()))


def set_comment(s, text):
    """the simflat_t's comment line (a 1024-byte buffer)"""
    b = text.encode()[:1023] + b"\0"
    field = C.addressof(s.contents) + type(s.contents).comment.offset
    buf = C.c_void_p.from_address(field).value  # the char* itself, not a copy
    if not buf:
        raise ValueError("simflat_t has no comment buffer")
    C.memmove(buf, b, len(b))


def print_it(s, path):
    """comdgb_printIt (printIt, write.c:89-110) into a file"""
    libc = C.CDLL(None)
    libc.fopen.restype = C.c_void_p
    libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
    libc.fclose.argtypes = [C.c_void_p]
    fp = libc.fopen(path.encode(), b"w")
    if not fp:
        raise OSError(f"cannot open {path}")
    try:
        load().comdgb_printIt(s, fp)
    finally:
        libc.fclose(fp)


def fcc(nx, ny, nz, lat, defgrad, bf, pot):
    """create_fcc_lattice on the host; returns a SimFlat pointer (caller frees)."""
    L = load()
    st = C.c_int(0)
    s = L.comdgb_fcc(nx, ny, nz, lat, defgrad, bf, pot.base, C.byref(st))
    if not s:
        raise ComdgbError(st.value, "comdgb_fcc failed: " + last_error())
    return s


def launch_probes(device=0):
    """(us per empty graph kernel node, us per grid-wide barrier)"""
    a, b = C.c_double(), C.c_double()
    check(load().comdgb_graph_node_cost(device, C.byref(a)))
    check(load().comdgb_grid_barrier_cost(device, C.byref(b)))
    return a.value, b.value


def rebin_host(s, bf):
    """comdgb_rebin_host: a new host simflat_t with the atoms of s binned at
    box factor bf (caller frees)"""
    st = C.c_int(0)
    out = load().comdgb_rebin_host(s, bf, C.byref(st))
    if not out:
        raise ComdgbError(st.value, "comdgb_rebin_host failed: " + last_error())
    return out


def batch_autotune(host_sims, o, box_factors=(), skins=(), steps=20, dt=1e-15,
                   cache_path=None):
    """comdgb_batch_autotune over the replicas; returns the Tune"""
    n = len(host_sims)
    arr = (P_SIM * n)(*host_sims)
    bfs = (C.c_double * max(len(box_factors), 1))(*box_factors)
    sks = (C.c_double * max(len(skins), 1))(*skins)
    t = Tune()
    check(load().comdgb_batch_autotune(arr, n, C.byref(o), bfs, len(box_factors), sks,
                                       len(skins), steps, dt,
                                       cache_path.encode() if cache_path else None,
                                       C.byref(t)))
    return t


def seed(s, seed_value, disp_kind, amp, temp_k, mass_amu):
    load().comdgb_seed(s, seed_value, disp_kind, amp, temp_k, mass_amu)


def free_host(s):
    load().comdgb_sim_free_host(s)


class DeviceSim:
    """A device-resident simulation handle (comdgb_sim_*)."""

    def __init__(self, host_sim, o):
        self.L = load()
        self.h = C.c_void_p()
        self._pot = o.potential
        self._nboxes = [host_sim.contents.nboxes]
        self._ntot = [host_sim.contents.ntot]
        check(self.L.comdgb_sim_create(host_sim, C.byref(o), C.byref(self.h)))

    def close(self):
        if self.h:
            self.L.comdgb_sim_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, s):
        check(self.L.comdgb_sim_upload(self.h, s))

    def download(self, s):
        check(self.L.comdgb_sim_download(self.h, s))

    def force(self):
        check(self.L.comdgb_sim_force(self.h))
        return self.energy()

    def steps(self, n, dt=1e-15):
        check(self.L.comdgb_sim_steps(self.h, n, dt))
        return self.energy()

    # ---- parameters and gradients (FP64 simulations) ----
    def _np(self, n):
        a = np.zeros(n, dtype=np.float64)
        return a, a.ctypes.data_as(C.POINTER(C.c_double))

    def nparams(self):
        return 2 if self._pot == POT_LJ else 96

    def get_cheby(self):
        c, pc = self._np(96)
        a, pa = self._np(3)
        b, pb = self._np(3)
        check(self.L.comdgb_sim_get_cheby(self.h, pc, pa, pb))
        return c, a, b

    def set_cheby(self, coef, x0, xn):
        c = np.ascontiguousarray(coef, dtype=np.float64)
        a = np.ascontiguousarray(x0, dtype=np.float64)
        b = np.ascontiguousarray(xn, dtype=np.float64)
        P = C.POINTER(C.c_double)
        check(self.L.comdgb_sim_set_cheby(self.h, c.ctypes.data_as(P), a.ctypes.data_as(P),
                                          b.ctypes.data_as(P)))

    def set_lj(self, epsilon, sigma):
        check(self.L.comdgb_sim_set_lj(self.h, epsilon, sigma))

    def energy_grad(self):
        """(U, dU/d(parameters))"""
        g, pg = self._np(self.nparams())
        e = C.c_double()
        check(self.L.comdgb_sim_energy_grad(self.h, C.byref(e), pg))
        return e.value, g

    def force_loss_grad(self, target):
        """(L, dL/d(parameters)) for L = sum |f_i - target[id_i]|^2"""
        t = np.ascontiguousarray(target, dtype=np.float64)
        g, pg = self._np(self.nparams())
        loss = C.c_double()
        check(self.L.comdgb_sim_force_loss_grad(self.h, t.ctypes.data_as(C.POINTER(C.c_double)),
                                                C.byref(loss), pg))
        return loss.value, g

    def traj_energy_grad(self, n, dt=1e-15, every=20):
        """(J, dJ/dc): J = potential energy after n steps"""
        g, pg = self._np(self.nparams())
        j = C.c_double()
        check(self.L.comdgb_sim_traj_energy_grad(self.h, n, dt, every, C.byref(j), pg))
        return j.value, g

    # ---- virial tensor and per-atom stress ----
    def virial(self):
        """force call and virial of every replica: (W[6], K[6], volume) of
        replica 0, Voigt order xx yy zz yz xz xy, Hartree (Angstrom^3)"""
        P = C.POINTER(C.c_double)
        w, k, v = np.zeros(6), np.zeros(6), C.c_double()
        check(self.L.comdgb_sim_virial(self.h, w.ctypes.data_as(P), k.ctypes.data_as(P),
                                       C.byref(v)))
        return w, k, v.value

    def atom_stress(self, r=0):
        """per-atom stress x volume of the last virial() call, replica r's slot
        layout: array [nboxes * 64, 6] (empty slots 0)"""
        a = np.zeros((self._nboxes[r] * 64, 6))
        check(self.L.comdgb_sim_atom_stress(self.h, r, a.ctypes.data_as(C.POINTER(C.c_double))))
        return a

    def centrosymmetry(self, r=0, approx=False):
        """(per-slot centrosymmetry of replica r [nboxes * 64], min, max)"""
        P = C.POINTER(C.c_double)
        out = np.zeros(self._nboxes[r] * 64)
        lo, hi = C.c_double(), C.c_double()
        check(self.L.comdgb_sim_centrosymmetry(self.h, r, int(approx), out.ctypes.data_as(P),
                                               C.byref(lo), C.byref(hi)))
        return out, lo.value, hi.value

    # ---- clsman output ----
    def gather(self, r=0):
        """replica r's atoms in id order: [ntot, 6] = position (box corner + r),
        momentum"""
        a = np.zeros((self._ntot[r], 6))
        check(self.L.comdgb_sim_gather(self.h, r, a.ctypes.data_as(C.POINTER(C.c_double))))
        return a

    def write_clsman(self, path, fmt=CLSMAN_BINARY, comment=None, r=0):
        check(self.L.comdgb_sim_write_clsman(self.h, r, path.encode(), fmt,
                                             None if comment is None else comment.encode()))

    def graph_steps(self, n, dt=1e-15):
        """n steps as one CUDA graph launch; returns its device time in ms"""
        ms = C.c_float()
        check(self.L.comdgb_sim_graph_steps(self.h, n, dt, C.byref(ms)))
        return ms.value

    def advance_velocity(self, dt):
        check(self.L.comdgb_sim_advance_velocity(self.h, dt))

    def advance_positions(self, dt):
        check(self.L.comdgb_sim_advance_positions(self.h, dt))

    def rebox(self):
        check(self.L.comdgb_sim_rebox(self.h))

    def energy(self):
        e, st = C.c_double(), C.c_double()
        check(self.L.comdgb_sim_energy(self.h, C.byref(e), C.byref(st)))
        return e.value, st.value

    def kinetic(self):
        ek = C.c_double()
        check(self.L.comdgb_sim_kinetic(self.h, C.byref(ek)))
        return ek.value

    def pair_count(self):
        v = C.c_longlong()
        check(self.L.comdgb_sim_pair_count(self.h, C.byref(v)))
        return v.value

    def synchronize(self):
        check(self.L.comdgb_sim_synchronize(self.h))

    def set_launch(self, build_threads=0, build_atoms=0, pass2_threads=0):
        """launch shapes of the force-order kernels (0: default)"""
        check(self.L.comdgb_sim_set_launch(self.h, build_threads, build_atoms, pass2_threads))

    def set_pair_table(self, on):
        """mixed EAM Chebyshev: pair functions from the FP32 segment table
        (True, default) or the FP32 series for every pair (False)"""
        check(self.L.comdgb_sim_set_pair_table(self.h, int(bool(on))))

    def set_list_capacity(self, cap):
        """neighbour-list entries per atom in use (0: as allocated); atoms
        beyond it scan their neighbour boxes"""
        check(self.L.comdgb_sim_set_list_capacity(self.h, cap))

    def apply_tune(self, t):
        """the launch shapes of a batch_autotune result"""
        check(self.L.comdgb_sim_apply_tune(self.h, C.byref(t)))

    def set_merge_rebox(self, on):
        """mixed precision: one rebox per step in a sequence of steps (default)
        or the reference's two (False)"""
        check(self.L.comdgb_sim_set_merge_rebox(self.h, int(bool(on))))

    def list_info(self):
        """(persistent lists in use, skin in A, persistent-list builds since upload)"""
        p, sk, n = C.c_int(), C.c_double(), C.c_longlong()
        check(self.L.comdgb_sim_list_info(self.h, C.byref(p), C.byref(sk), C.byref(n)))
        return bool(p.value), sk.value, n.value

    def step_launches(self, n):
        """kernels a sequence of n steps launches"""
        v = C.c_longlong()
        check(self.L.comdgb_sim_step_launches(self.h, n, C.byref(v)))
        return v.value

    def rebuild_launches(self):
        """kernels of a step's rebuild section, launched once per list
        rebuild (0 when the rebuild section is not a conditional node)"""
        v = C.c_int()
        check(self.L.comdgb_sim_rebuild_launches(self.h, C.byref(v)))
        return v.value

    def graph_kernels(self):
        a, b = C.c_int(), C.c_int()
        check(self.L.comdgb_sim_graph_kernels(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def timed_steps(self, n, dt=1e-15, max_kernels=16):
        """(per-step ms, span ms, {kernel group: mean ms per step})"""
        step = (C.c_float * (n + 1))()
        kern = (C.c_float * max_kernels)()
        nk = check(self.L.comdgb_sim_timed_steps(self.h, n, dt, step, kern, max_kernels))
        names = [self.L.comdgb_kernel_name(self.h, k).decode() for k in range(nk)]
        return list(step)[:n], step[n], dict(zip(names, list(kern)[:nk]))


class Batch(DeviceSim):
    """Replicas advanced together (comdgb_batch_*): the DeviceSim calls act on
    all of them; uploads, downloads and energies go per replica."""

    def __init__(self, host_sims, o):
        self.L = load()
        self.h = C.c_void_p()
        self._pot = o.potential
        self.n = len(host_sims)
        self._nboxes = [q.contents.nboxes for q in host_sims]
        self._ntot = [q.contents.ntot for q in host_sims]
        arr = (P_SIM * self.n)(*host_sims)
        check(self.L.comdgb_batch_create(arr, self.n, C.byref(o), C.byref(self.h)))

    def upload_rep(self, r, s):
        check(self.L.comdgb_batch_upload(self.h, r, s))

    def download_rep(self, r, s):
        check(self.L.comdgb_batch_download(self.h, r, s))

    def energies(self):
        e = np.zeros(self.n)
        st = np.zeros(self.n)
        P = C.POINTER(C.c_double)
        check(self.L.comdgb_batch_energies(self.h, e.ctypes.data_as(P), st.ctypes.data_as(P)))
        return e, st

    def virial_rep(self, r):
        """replica r's (W, K, volume) of the last virial() call"""
        P = C.POINTER(C.c_double)
        w, k, v = np.zeros(6), np.zeros(6), C.c_double()
        check(self.L.comdgb_batch_virial(self.h, r, w.ctypes.data_as(P), k.ctypes.data_as(P),
                                         C.byref(v)))
        return w, k, v.value
