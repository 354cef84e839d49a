"""CPU tests of the library's host side: the shared library loads and exports
every entry point of include/comdgb.h, the host setup routines reproduce
the oracle's byte for byte, GPU calls fail with an error code (never a CPU
fallback) when no GPU is present, and the replica path of bench.py works
across two gloo ranks."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import comd_gb300 as cg
from comd_gb300.abi import slot_views

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "comdgb.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(comdgb_\w+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    lib = cg.load()
    names = declared_symbols()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_tables_match_oracle(oracle, pots_dir):
    pot = cg.eam_potential("cu")
    opot = oracle.eam(pots_dir, "cu")
    for name in ("phi", "rho", "f"):
        a = getattr(pot.ptr.contents, name).contents
        b = getattr(opot.contents, name).contents
        assert (a.n, a.x0, a.xn, a.invDx) == (b.n, b.x0, b.xn, b.invDx)
        va = np.ctypeslib.as_array(C.cast(C.addressof(a.values.contents) - 8,
                                          C.POINTER(C.c_double)), (a.n + 3,))
        vb = np.ctypeslib.as_array(C.cast(C.addressof(b.values.contents) - 8,
                                          C.POINTER(C.c_double)), (b.n + 3,))
        assert np.array_equal(va, vb)
    assert pot.ptr.contents.mass == 63.55 and pot.ptr.contents.lat == 3.615
    assert pot.ptr.contents.cutoff == 4.961


@pytest.mark.parametrize("dims", [(10, 10, 10, 1.0, 1.0), (13, 13, 13, 1.05, 1.5),
                                  (3, 5, 2, 1.0, 1.0)])
def test_fcc_and_seed_match_oracle(oracle, pots_dir, dims):
    nx, ny, nz, dg, bf = dims
    pot = cg.eam_potential("cu")
    opot = oracle.eam(pots_dir, "cu")
    s = cg.fcc(nx, ny, nz, 3.615, dg, bf, pot)
    so = oracle.fcc(nx, ny, nz, 3.615, dg, bf, opot)
    cg.seed(s, 99, cg.DISP_GAUSSIAN, 0.05, 600.0, 63.55)
    oracle.seed(so, 99, cg.DISP_GAUSSIAN, 0.05, 600.0, 63.55)
    assert list(s.contents.nbx) == list(so.contents.nbx)
    assert s.contents.ntot == so.contents.ntot == 4 * nx * ny * nz
    va, vb = slot_views(s), slot_views(so)
    for k in va:
        assert np.array_equal(va[k], vb[k]), k
    cg.free_host(s)
    oracle.free(so)


def test_seed_momenta_have_zero_total(oracle, pots_dir):
    pot = oracle.eam(pots_dir, "cu")
    s = oracle.fcc(6, 6, 6, 3.615, 1.0, 1.0, pot)
    oracle.seed(s, 3, 0, 0.0, 300.0, 63.55)
    v = slot_views(s)
    m = np.arange(64)[None, :] < v["natoms"][:, None]
    p = v["p"][m.reshape(-1)]
    assert np.abs(p.sum(0)).max() < 1e-9 * np.abs(p).max()
    # equipartition: <p^2/2M> = 3/2 kT within sampling error
    ek = (p ** 2).sum() / (2 * 63.55 * 1822.83)
    kt = 3.166811563e-6 * 300.0
    assert abs(ek / (1.5 * kt * len(p)) - 1) < 0.1
    oracle.free(s)


def test_gpu_entry_points_fail_loudly_without_gpu():
    """Without a usable GPU the library returns an error; it never computes on the CPU."""
    import subprocess
    import sys
    code = (
        "import os, sys; sys.path.insert(0, %r); os.environ['CUDA_VISIBLE_DEVICES'] = '';"
        "import comd_gb300 as cg\n"
        "pot = cg.eam_potential('cu'); s = cg.fcc(4, 4, 4, 3.615, 1, 1, pot)\n"
        "try:\n    cg.DeviceSim(s, cg.opts()); print('CREATED')\n"
        "except cg.ComdgbError as e:\n    print('ERR', e.code)\n" % ROOT)
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True,
                         env=dict(os.environ, CUDA_VISIBLE_DEVICES=""), timeout=120)
    assert "ERR" in out.stdout, out.stdout + out.stderr
    assert "CREATED" not in out.stdout


def _replica_rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import sys
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist(world)
    d.barrier()
    s = d.sum(rank + 1.0)
    m = d.max(10.0 * rank)
    d.close()
    q.put((rank, s, m))


def test_bench_replicas_over_gloo():
    """bench.py's N>1 path (replicas): barrier, sum of work and max of time over 2 ranks."""
    pytest.importorskip("torch")
    import multiprocessing as mp
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_replica_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
    assert res == [(0, 3.0, 10.0), (1, 3.0, 10.0)]


def test_round_f32_matches_ieee_nearest_even():
    """The integer FP64 -> FP32 rounding of the mixed-precision positions
    equals IEEE round-to-nearest-even (numpy's conversion), ties included."""
    rng = np.random.default_rng(7)
    x = np.concatenate([rng.uniform(-4.0, 4.0, 200000),
                        rng.uniform(0.0, 1e-3, 1000), rng.normal(0.0, 1e3, 1000),
                        [0.0, -0.0, 1.0, -1.0, 3.4e38, 1e-40, -1e-45, 1e300, np.inf, -np.inf]])
    # exact ties: FP32 values plus half an FP32 ulp (representable in FP64)
    f = rng.uniform(0.5, 4.0, 5000).astype(np.float32)
    ulp = np.spacing(f).astype(np.float64)
    x = np.concatenate([x, f.astype(np.float64) + 0.5 * ulp, f.astype(np.float64) - 0.5 * ulp])
    with np.errstate(over="ignore"):
        want = x.astype(np.float32)
    got = cg.round_f32(x)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    nan = cg.round_f32(np.array([np.nan]))
    assert np.isnan(nan[0])


def _write_table(path, n, x0, xn, invdx, rec=None, values=None, big_endian=True):
    """a table file in the reference's Fortran-record layout (eam.c:156-249)"""
    import struct
    e = ">" if big_endian else "<"
    vals = np.linspace(1.0, 0.0, n) if values is None else values
    with open(path, "wb") as f:
        f.write(struct.pack(e + "i", 36))
        f.write(struct.pack(e + "idddii", n, x0, xn, invdx, 1, 0))
        f.write(struct.pack(e + "ii", 36, 8 * n if rec is None else rec))
        f.write(struct.pack(e + "%dd" % len(vals), *vals))
        f.write(struct.pack(e + "i", 8 * n))


@pytest.mark.parametrize("case", ["good", "good_le", "truncated", "zero_n", "bad_record",
                                  "nan_x0", "empty_range", "zero_invdx", "inf_invdx"])
def test_eam_read_rejects_malformed_tables(tmp_path, case):
    """comdgb_eam_read loads a table only when the interpolation can index it:
    n > 0 values, x0 < xn finite, 1/dx finite and positive, a data record of
    8n bytes; a short file is rejected too.  Either byte order is read."""
    import shutil
    for ext in ("rho", "f", "doc"):
        shutil.copy(os.path.join(cg.POT_DIR, "cu." + ext), tmp_path / ("t." + ext))
    n, x0, xn = 3000, 1.0, 4.961
    invdx = n / (xn - x0)
    args = {"good": (n, x0, xn, invdx), "good_le": (n, x0, xn, invdx),
            "truncated": (n, x0, xn, invdx), "zero_n": (0, x0, xn, invdx),
            "bad_record": (n, x0, xn, invdx), "nan_x0": (n, float("nan"), xn, invdx),
            "empty_range": (n, xn, xn, invdx), "zero_invdx": (n, x0, xn, 0.0),
            "inf_invdx": (n, x0, xn, float("inf"))}[case]
    phi = str(tmp_path / "t.phi")
    _write_table(phi, *args, rec=8 * n + 8 if case == "bad_record" else None,
                 values=np.linspace(1.0, 0.0, 0 if case == "zero_n" else n),
                 big_endian=case != "good_le")
    if case == "truncated":
        with open(phi, "r+b") as f:
            f.truncate(48 + 8 * 100)
    L = cg.load()
    p = L.comdgb_eam_read(str(tmp_path).encode(), b"t")
    if case.startswith("good"):
        assert p, case
        a = p.contents.phi.contents
        assert (a.n, a.xn, a.invDx) == (n, xn, invdx)
        L.comdgb_eam_free(p)
    else:
        assert not p, case
        assert "t.phi" in cg.lib.last_error(), cg.lib.last_error()


def test_host_binning_rejects_non_finite_and_far_coordinates(tmp_path):
    """Host binning (comdgb_read_clsman with device < 0, the path of
    putAtomInBox on the host) gives COMDGB_ERR_BOXRANGE for a NaN or
    infinite coordinate and for an atom more than one period outside, on
    every host (the int conversion of floor(NaN) is host-dependent), as the
    device binning does; an atom less than one period outside is wrapped."""
    pot = cg.eam_potential("cu")

    def clsman(x):
        p = tmp_path / "one.inp"
        p.write_text("2 0\ncomment\n21.69 21.69 21.69\n"
                     "1.0 1.0 1.0 0 0.0 0.0 0.0\n%s 2.0 2.0 0 0.0 0.0 0.0\n" % x)
        return str(p)

    s = cg.read_clsman(clsman("-1.5"), pot, 1.0, -1)  # wrapped into the period
    try:
        assert s.contents.ntot == 2
    finally:
        cg.free_host(s)
    for bad in ("nan", "inf", "-inf", "-30.0", "50.0"):
        with pytest.raises(cg.ComdgbError) as ei:
            cg.read_clsman(clsman(bad), pot, 1.0, -1)
        assert ei.value.code == -12, bad  # COMDGB_ERR_BOXRANGE
        assert "one.inp" in str(ei.value) and "not finite" in str(ei.value), str(ei.value)


def test_clsman_count_beyond_the_file_is_an_io_error(tmp_path):
    """an atom count that the file cannot hold fails before any allocation
    for it (no multi-gigabyte request from a corrupt header)"""
    pot = cg.eam_potential("cu")
    p = tmp_path / "huge.inp"
    p.write_text("2000000000 0\ncomment\n21.69 21.69 21.69\n1.0 1.0 1.0 0 0.0 0.0 0.0\n")
    with pytest.raises(cg.ComdgbError) as ei:
        cg.read_clsman(str(p), pot, 1.0, -1)
    assert ei.value.code == -33  # COMDGB_ERR_IO
    assert "huge.inp" in str(ei.value), str(ei.value)


@pytest.mark.parametrize("nbx", [(64, 64, 8), (2**31 - 1,) * 3, (128, 128, 2**31 - 1)])
def test_noalloc_binning_rejects_grids_beyond_its_scratch_without_a_gpu(nbx):
    """comdgb_put_atoms_noalloc checks the grid against its fixed scratch
    (16,384 boxes) before any CUDA call, with no integer overflow for the
    largest int extents"""
    L = cg.load()
    n3 = (C.c_int * 3)(*nbx)
    bounds = (C.c_double * 3)(100.0, 100.0, 100.0)
    bs = (C.c_double * 3)(*(100.0 / k for k in nbx))
    dummy = C.c_void_p(1)
    rc = L.comdgb_put_atoms_noalloc(n3, bounds, bs, dummy, 0, None, None, None, None, None,
                                    dummy, dummy, dummy, dummy, dummy, dummy, 0, None)
    assert rc == -1  # COMDGB_ERR_ARG
    assert "allocation-free limit" in cg.lib.last_error()


def test_grid_beyond_int_slot_indexes_is_an_argument_error():
    """allocDomains' grid (domains.c:155-200) for a lattice whose slot
    indexes (box * 64 + k) would not fit an int is refused with
    COMDGB_ERR_ARG before anything is allocated; a grid below one box per
    axis keeps the reference's -3"""
    pot = cg.eam_potential("cu")
    # 728^3 = 386 M boxes and 72,868^3 (an int product that overflows) against
    # the 33.5 M boxes whose slot indexes fit an int
    for n in (1000, 100000):
        with pytest.raises(cg.ComdgbError) as ei:
            cg.fcc(n, n, n, 3.615, 1.0, 1.0, pot)
        assert ei.value.code == -1, n  # COMDGB_ERR_ARG
        assert "slot indexes" in cg.lib.last_error()
    with pytest.raises(cg.ComdgbError) as ei:
        cg.fcc(1, 1, 1, 3.615, 1.0, 1.0, pot)  # 3.615 A < the 4.961 A cutoff
    assert ei.value.code == -3  # COMDGB_ERR_NOBOX


def test_create_checks_the_box_grid_before_any_cuda_call():
    """comdgb_sim_create / comdgb_attach refuse a simflat_t whose nboxes is not
    nbx[0]*nbx[1]*nbx[2], or whose box sizes are unset, with COMDGB_ERR_ARG
    (before touching the GPU; the stencil kernels index boxes by nbx)"""
    L = cg.load()
    pot = cg.eam_potential("cu")
    s = cg.fcc(6, 6, 6, 3.615, 1.0, 1.0, pot)
    o = cg.opts()
    h = C.c_void_p()
    try:
        nb = s.contents.nboxes
        s.contents.nboxes = nb + 1
        assert L.comdgb_sim_create(s, C.byref(o), C.byref(h)) == -1
        assert "nboxes" in cg.lib.last_error()
        assert L.comdgb_attach(s, C.byref(o)) == -1
        s.contents.nboxes = nb
        bs = s.contents.boxsize[1]
        s.contents.boxsize[1] = float("nan")
        assert L.comdgb_sim_create(s, C.byref(o), C.byref(h)) == -1
        s.contents.boxsize[1] = bs
    finally:
        cg.free_host(s)


def _c_kind(decl):
    """'int', 'long', 'long long', 'double', 'float', 'uint64', 'void' or
    'ptr' for one C parameter or return declaration of include/comdgb.h"""
    d = " ".join(decl.replace("const", " ").split())
    if "*" in d or "[" in d:
        return "ptr"
    words = d.split()
    base = " ".join(w for w in words[:-1]) if len(words) > 1 else words[0]
    return {"int": "int", "long": "long", "long long": "long long", "double": "double",
            "float": "float", "uint64_t": "uint64", "void": "void", "size_t": "ulong"}[base]


def _py_kind(t):
    if t is None:
        return "void"
    for ct, k in ((C.c_int, "int"), (C.c_double, "double"), (C.c_float, "float"),
                  (C.c_uint64, "uint64"), (C.c_longlong, "long long"), (C.c_long, "long")):
        if t is ct:
            return k
    if t in (C.c_void_p, C.c_char_p) or hasattr(t, "_type_") and issubclass(t, C._Pointer):
        return "ptr"
    raise AssertionError(f"unclassified ctypes type {t}")


def test_binding_prototypes_match_the_header():
    """Every entry point the Python binding declares (argtypes) takes the
    parameters and returns the type include/comdgb.h gives it, kind for kind
    (a double passed where the C side reads an int would not be caught by
    ctypes), so the tests call the library as a C caller would."""
    src = open(os.path.join(ROOT, "include", "comdgb.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    protos = {}
    for m in re.finditer(r"([A-Za-z_][\w \*]*?)\b(comdgb_\w+)\s*\(([^)]*)\)\s*;", src):
        ret, name, params = m.group(1), m.group(2), m.group(3).strip()
        args = [] if params in ("", "void") else [_c_kind(p) for p in params.split(",")]
        protos[name] = (_c_kind(ret.strip() + " x"), args)
    lib = cg.load()
    checked = 0
    for name, (ret, args) in protos.items():
        fn = getattr(lib, name)
        if fn.argtypes is None:
            continue
        # long and long long are one ctypes type where they have one size
        same = C.sizeof(C.c_long) == C.sizeof(C.c_longlong)
        canon = (lambda k: "long long" if same and k == "long" else k)
        assert [canon(_py_kind(t)) for t in fn.argtypes] == [canon(a) for a in args], name
        want = "int" if fn.restype is C.c_int else _py_kind(fn.restype)
        # a void function's ctypes default (int) result is never read
        assert want == ret or (ret == "void" and want == "int"), (name, want, ret)
        checked += 1
    assert checked >= 70, checked
