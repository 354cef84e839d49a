"""clsman output (write.c:112-220) and printIt (write.c:89-110).

The reference's own writers, run on the same states by
tests/golden/make_golden.py, give sha256 digests of the binary file
(writeClsman), of the decompressed text (gzASCIIWrite) and of printIt's
output.  The library's files must match them byte for byte: from a host
simflat_t (host gather) on CPU, and from device state (device gather by id)
on the GPU.  The gzip bytes themselves differ (several gzip members instead
of one stream); what a reader gets back is identical."""
import ctypes as C
import gzip
import hashlib
import os

import numpy as np
import pytest

import comd_gb300 as cg
from comd_gb300.abi import by_id, slot_views
from helpers import FIX
from oracle import KIND_EAM_TABLE

WFIX = FIX["clsman_writers"]
SEEDED_COMMENT = "seeded Cu lattice 6x6x6\n"


def sha(b):
    return hashlib.sha256(b).hexdigest()


def digests(binary_path, text_gz_path):
    return sha(open(binary_path, "rb").read()), sha(gzip.open(text_gz_path).read())


AG = {}


def ag8k_host():
    """the Ag 8k file as read (its atoms are already in their boxes, so the
    reBoxAll of initSimFromCmdLine moves nothing); the potential is kept for
    the module's lifetime (the simulation points at it)"""
    pot = AG.setdefault("pot", cg.eam_potential("ag"))
    return cg.read_clsman(os.path.join(cg.DATA_DIR, "8k.inp.gz"), pot, 1.0, -1)


def seeded_cu_host(oracle):
    """the seeded 6^3 Cu lattice of the fixture, reboxed and with the
    reference's table forces (the oracle's, bit for bit)"""
    pot = cg.eam_potential("cu")
    s = cg.fcc(6, 6, 6, pot.ptr.contents.lat, 1.0, 1.0, pot)
    cg.seed(s, 21, cg.DISP_GAUSSIAN, 0.05, 600.0, 63.55)
    assert oracle.rebox(s) == 0
    assert oracle.force(s, KIND_EAM_TABLE) == 0
    cg.set_comment(s, SEEDED_COMMENT)
    return s, pot


def gzip_available():
    s = ag8k_host()
    cg.free_host(s)
    return True


@pytest.fixture(scope="module")
def have_zlib():
    try:
        return gzip_available()
    except cg.ComdgbError as e:
        if e.code == -34:
            return False
        raise


# ---------------------------------------------------------------- CPU ----

def test_host_writers_match_reference_ag8k(tmp_path, have_zlib):
    if not have_zlib:
        pytest.skip("library built without zlib")
    s = ag8k_host()
    try:
        cg.write_clsman_host(s, str(tmp_path / "a.bin"), True)
        cg.write_clsman_host(s, str(tmp_path / "a.txt.gz"), False)
        cg.print_it(s, str(tmp_path / "a.print"))
        fb, ft = digests(tmp_path / "a.bin", tmp_path / "a.txt.gz")
        ref = WFIX["ag8k_read"]
        assert (fb, ft) == (ref["binary_sha256"], ref["text_sha256"])
        assert sha(open(tmp_path / "a.print", "rb").read()) == ref["print_sha256"]
    finally:
        cg.free_host(s)


def test_host_writers_match_reference_seeded(oracle, tmp_path, have_zlib):
    if not have_zlib:
        pytest.skip("library built without zlib")
    s, _pot = seeded_cu_host(oracle)
    try:
        cg.write_clsman_host(s, str(tmp_path / "c.bin"), True)
        cg.write_clsman_host(s, str(tmp_path / "c.txt.gz"), False)
        cg.print_it(s, str(tmp_path / "c.print"))
        ref = WFIX["cu6_seeded_forced"]
        assert digests(tmp_path / "c.bin", tmp_path / "c.txt.gz") == (ref["binary_sha256"],
                                                                      ref["text_sha256"])
        assert sha(open(tmp_path / "c.print", "rb").read()) == ref["print_sha256"]
        assert os.path.getsize(tmp_path / "c.bin") == ref["binary_bytes"]
    finally:
        cg.free_host(s)


def test_binary_layout(oracle, tmp_path):
    """the record structure of writeClsman, field by field"""
    s, _pot = seeded_cu_host(oracle)
    try:
        cg.write_clsman_host(s, str(tmp_path / "c.bin"), True)
        b = open(tmp_path / "c.bin", "rb").read()
        n = s.contents.ntot
        head = np.frombuffer(b[:28], dtype=np.int32)
        assert list(head) == [12, n, 0, 0, 12, 0, 0]
        assert np.frombuffer(b[28:32], np.int32)[0] == 24
        assert list(np.frombuffer(b[32:56], np.float64)) == list(s.contents.bounds)
        assert np.frombuffer(b[56:64], np.int32).tolist() == [24, 52 * n]
        rec = np.frombuffer(b[64:64 + 52 * n], dtype=np.dtype(
            [("x", "<f8", 3), ("t", "<i4"), ("p", "<f8", 3)]))
        assert np.frombuffer(b[64 + 52 * n:], np.int32).tolist() == [52 * n]
        assert np.array_equal(rec["x"], world_by_id(s))
        assert np.all(rec["t"] == 1)
        assert np.array_equal(rec["p"], by_id(s, "p"))
    finally:
        cg.free_host(s)


def test_text_round_trip(oracle, tmp_path):
    """a text file the library writes reads back (fromFileASCII's format):
    same atom count and bounds, positions and momenta to the 1e-8 of %.8lf"""
    s, pot = seeded_cu_host(oracle)
    try:
        txt = write_plain_text_host(s, str(tmp_path / "c.txt"))
        back = cg.read_clsman(txt, pot, 1.0, -1)
        try:
            assert back.contents.ntot == s.contents.ntot
            assert np.allclose(list(back.contents.bounds), list(s.contents.bounds), atol=1e-8)
            xa = world_by_id(s)
            xb = world_by_id(back)
            assert np.abs(xa - xb).max() <= 0.6e-8
            assert np.abs(by_id(s, "p") - by_id(back, "p")).max() <= 0.6e-8
            assert open(txt).read().splitlines()[1] == SEEDED_COMMENT.strip()
        finally:
            cg.free_host(back)
    finally:
        cg.free_host(s)


def write_plain_text_host(s, path):
    """plain-text output of a host simflat_t: gzASCIIWrite's lines, written by
    decompressing the drop-in's gzip file when zlib is there, else formatted
    here as the reference formats them"""
    try:
        cg.write_clsman_host(s, path + ".gz", False)
        open(path, "wb").write(gzip.open(path + ".gz").read())
    except cg.ComdgbError as e:
        if e.code != -34:
            raise
        x, p = world_by_id(s), by_id(s, "p")
        b = s.contents.bounds
        with open(path, "w") as f:
            f.write(f"{s.contents.ntot} 0\n{SEEDED_COMMENT}")
            f.write("%.8f %.8f %.8f\n" % (b[0], b[1], b[2]))
            for q in range(len(x)):
                f.write("%.8f %.8f %.8f 1 %.8f %.8f %.8f\n" % (*x[q], *p[q]))
    return path


def world_by_id(s):
    v = slot_views(s)
    n = s.contents.ntot
    occ = (np.arange(64)[None, :] < v["natoms"][:, None]).reshape(-1)
    world = (np.repeat(v["dcenter"], 64, axis=0) + v["r"])[occ]
    out = np.empty((n, 3))
    out[v["id"][occ]] = world
    return out


def test_duplicate_id_is_an_error(oracle, tmp_path):
    """getRL reports a duplicated or missing id and writes anyway; the
    library refuses (COMDGB_ERR_ARG) and writes nothing"""
    s, _pot = seeded_cu_host(oracle)
    try:
        v = slot_views(s)
        v["id"][1] = v["id"][0]
        with pytest.raises(cg.ComdgbError) as e:
            cg.write_clsman_host(s, str(tmp_path / "d.bin"), True)
        assert e.value.code == -1
        assert not os.path.exists(tmp_path / "d.bin")
    finally:
        cg.free_host(s)


def test_empty_comment_writes_an_empty_line(tmp_path, have_zlib):
    """gzASCIIWrite exits (-98) on an empty comment (a generated lattice's);
    the library writes an empty comment line so the file reads back"""
    if not have_zlib:
        pytest.skip("library built without zlib")
    pot = cg.eam_potential("cu")
    s = cg.fcc(3, 3, 3, pot.ptr.contents.lat, 1.0, 1.0, pot)
    try:
        cg.write_clsman_host(s, str(tmp_path / "e.txt.gz"), False)
        lines = gzip.open(tmp_path / "e.txt.gz").read().decode().split("\n")
        assert lines[0] == f"{s.contents.ntot} 0" and lines[1] == ""
        back = cg.read_clsman(str(tmp_path / "e.txt.gz"), pot, 1.0, -1)
        assert back.contents.ntot == s.contents.ntot
        cg.free_host(back)
    finally:
        cg.free_host(s)


# ---------------------------------------------------------------- GPU ----

@pytest.mark.gpu
def test_device_writers_match_reference(oracle, tmp_path):
    for name, make in (("ag8k_read", lambda: (ag8k_host(), None)),
                       ("cu6_seeded_forced", lambda: seeded_cu_host(oracle))):
        s, _pot = make()
        try:
            d = cg.DeviceSim(s, cg.opts(cg.POT_EAM_TABLE, cg.PREC_FP64))
            try:
                comment = C.string_at(s.contents.comment).decode()
                d.write_clsman(str(tmp_path / "d.bin"), cg.CLSMAN_BINARY)
                d.write_clsman(str(tmp_path / "d.txt.gz"), cg.CLSMAN_TEXT_GZ, comment)
                d.write_clsman(str(tmp_path / "d.txt"), cg.CLSMAN_TEXT, comment)
                g = d.gather()
            finally:
                d.close()
            ref = WFIX[name]
            assert digests(tmp_path / "d.bin", tmp_path / "d.txt.gz") == (ref["binary_sha256"],
                                                                          ref["text_sha256"])
            assert sha(open(tmp_path / "d.txt", "rb").read()) == ref["text_sha256"]
            assert np.array_equal(g[:, :3], world_by_id(s))
            assert np.array_equal(g[:, 3:], by_id(s, "p"))
        finally:
            cg.free_host(s)


@pytest.mark.gpu
def test_attached_dropin_writes_device_state(oracle, tmp_path):
    s, _pot = seeded_cu_host(oracle)
    L = cg.load()
    try:
        o = cg.opts(cg.POT_EAM_TABLE, cg.PREC_FP64)
        assert L.comdgb_attach(s, C.byref(o)) == 0
        try:
            assert L.comdgb_set_lazy(s, 1) == 0  # the device holds the state
            assert L.comdgb_writeClsman(s, str(tmp_path / "a.bin").encode()) == 0
            assert L.comdgb_gzASCIIWrite(s, str(tmp_path / "a.txt.gz").encode()) == 0
        finally:
            L.comdgb_detach(s)
        ref = WFIX["cu6_seeded_forced"]
        assert digests(tmp_path / "a.bin", tmp_path / "a.txt.gz") == (ref["binary_sha256"],
                                                                      ref["text_sha256"])
    finally:
        cg.free_host(s)


@pytest.mark.gpu
def test_device_write_after_steps_equals_host_write(oracle, tmp_path):
    """after 10 mixed-precision steps: the device gather and the host gather
    of the downloaded state write the same bytes"""
    s, _pot = seeded_cu_host(oracle)
    try:
        d = cg.DeviceSim(s, cg.opts(cg.POT_EAM_CHEBY, cg.PREC_MIXED))
        try:
            d.steps(10)
            d.write_clsman(str(tmp_path / "d.bin"))
            d.write_clsman(str(tmp_path / "d.txt"), cg.CLSMAN_TEXT, SEEDED_COMMENT)
            d.download(s)
        finally:
            d.close()
        cg.write_clsman_host(s, str(tmp_path / "h.bin"), True)
        assert open(tmp_path / "d.bin", "rb").read() == open(tmp_path / "h.bin", "rb").read()
        txt = write_plain_text_host(s, str(tmp_path / "h.txt"))
        assert open(tmp_path / "d.txt", "rb").read() == open(txt, "rb").read()
    finally:
        cg.free_host(s)


@pytest.mark.gpu
def test_batch_replica_write_equals_single(tmp_path):
    from test_batch import make_replicas
    pot = cg.eam_potential("cu")
    o = cg.opts(cg.POT_EAM_CHEBY, cg.PREC_FP64, True, per_step_lists=True)
    bs, ss = make_replicas(pot), make_replicas(pot)
    try:
        b = cg.Batch(bs, o)
        try:
            b.steps(5)
            for r in range(b.n):
                b.write_clsman(str(tmp_path / f"b{r}.bin"), cg.CLSMAN_BINARY, None, r)
        finally:
            b.close()
        for r, s in enumerate(ss):
            d = cg.DeviceSim(s, o)
            try:
                d.steps(5)
                d.write_clsman(str(tmp_path / f"s{r}.bin"))
            finally:
                d.close()
            assert open(tmp_path / f"b{r}.bin", "rb").read() == \
                open(tmp_path / f"s{r}.bin", "rb").read(), r
    finally:
        for s in bs + ss:
            cg.free_host(s)
