"""The drop-in boundary driven from C.

comd_gb300/comdgb_run is host/comdgb_run.c linked with -lcomdgb: the
reference's set-up (initSimFromCmdLine, src-flat/docompute.c:68-163) and
timestep loop (do_compute_work, :166-218) with `sim->pot->force =
comdgb_force` and comdgb_nTimeSteps in place of nTimeSteps.  The GPU test
runs it on a seeded EAM Cu Chebyshev lattice and compares the energy it
prints after the initial force call and after every nTimeSteps(10) with the
oracle running the same loop on the same state: FP64 to 1e-10 relative,
mixed precision to 1e-7 Ha per atom.
"""
import json
import os
import re
import subprocess

import pytest

import comd_gb300 as cg
from comd_gb300.build import HOST_OUT, INCLUDE, OUT, build
from helpers import Case

LINE = re.compile(r"^\s*(\d+)\s+(\S+)\s+computed in")


def _run_host(args):
    build()
    r = subprocess.run([HOST_OUT] + args, capture_output=True, text=True, timeout=600)
    return r


def test_host_links_against_library():
    """the binary starts (the dynamic linker finds libcomdgb.so) and prints
    its usage without touching a GPU"""
    r = _run_host(["-h"])
    assert r.returncode == 2, r.stderr
    assert "usage" in r.stderr


def test_host_without_a_gpu_fails_with_the_library_error():
    """without a usable GPU the C host stops at its first GPU call (the
    Chebyshev fit) with exit status 1 and the library's message; nothing is
    computed on the CPU"""
    build()
    r = subprocess.run([HOST_OUT, "-e", "-c", "-p", "cu", "-d", cg.POT_DIR, "-x", "4", "-y", "4",
                        "-z", "4", "-m"], capture_output=True, text=True, timeout=300,
                       env=dict(os.environ, CUDA_VISIBLE_DEVICES=""))
    assert r.returncode == 1, r.stdout + r.stderr
    m = re.search(r"comdgb_cheb_make failed \(-30\): (.+)", r.stderr)
    assert m and m.group(1).strip(), r.stderr
    assert "Starting simulation" not in r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("mixed", [False, True])
def test_host_loop_matches_oracle(oracle, mixed):
    n, niter, nsteps, seed, temp, amp = 8, 3, 10, 7, 600.0, 0.05
    args = ["-e", "-c", "-p", "cu", "-d", cg.POT_DIR, "-x", str(n), "-y", str(n), "-z", str(n),
            "-t", str(temp), "-a", str(amp), "-S", str(seed), "-n", str(niter), "-k",
            str(nsteps)] + (["-m"] if mixed else [])
    r = _run_host(args)
    assert r.returncode == 0, r.stdout + r.stderr
    got = [(int(m.group(1)), float(m.group(2))) for m in map(LINE.match, r.stdout.splitlines())
           if m]
    assert [s for s, _ in got] == [nsteps * i for i in range(niter + 1)], r.stdout
    c = Case(oracle, cg.POT_EAM_CHEBY, n=(n, n, n), seed=seed, disp=cg.DISP_GAUSSIAN, amp=amp,
             temp=temp)
    try:
        ntot = c.s.contents.ntot
        c.oracle_force()
        want = [c.o.contents.e]
        for _ in range(niter):
            assert c.oracle.steps(c.o, nsteps, 1e-15, c.kind) == 0
            want.append(c.o.contents.e)
    finally:
        c.close()
    for (step, e), eo in zip(got, want):
        if mixed:
            assert abs(e - eo) / ntot < 1e-7, (step, e, eo)
        else:
            assert abs(e - eo) <= 1e-10 * abs(eo), (step, e, eo)
    # the run's JSON record agrees with the printed lines
    rec = [json.loads(l)["comdgb_run"] for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(rec) == 1, r.stdout
    assert rec[0]["atoms"] == ntot and rec[0]["iterations"] == niter
    assert rec[0]["precision"] == ("mixed" if mixed else "fp64")
    assert rec[0]["final_energy"] == got[-1][1] and rec[0]["atom_steps_per_s"] > 0


# The maintainer's edits of INTEGRATION.md, taken from the document itself
# and applied to copies of the reference's own sources in a temporary
# directory (nothing of the reference is kept): comdgb.h after pmd.h, the
# attach and the force pointer at the end of initSimFromCmdLine (item 1),
# comdgb_nTimeSteps in do_compute_work's loop (item 2), the detach before
# destroySimulation (item 4) and the clsman reader (item 8).
def _integration_snippets():
    text = open(os.path.join(os.path.dirname(INCLUDE), "INTEGRATION.md")).read()
    sec = text.split("## What a maintainer adds to the reference", 1)[1]
    attach = re.search(r"```c\n(.*?)```", sec, re.S).group(1)
    read = re.search(r"```c\n(.*?)```", sec.split("8. Structure files", 1)[1], re.S).group(1)
    includes = "".join(l + "\n" for l in attach.splitlines() if l.startswith("#include"))
    attach = "".join(l + "\n" for l in attach.splitlines() if not l.startswith("#include"))
    return includes, attach, read


def _edit(text, old, new):
    assert text.count(old) == 1, old
    return text.replace(old, new)


def test_reference_program_builds_with_the_documented_edits(tmp_path):
    """The reference's own program (src-flat: pmd.c's main, initSimFromCmdLine
    and do_compute_work) compiles and links against libcomdgb with the edits
    INTEGRATION.md lists, its C snippets pasted as written, with pointer
    types checked as errors: comdgb.h then uses the reference's own struct
    definitions.  Run without a GPU it gets through the reference's set-up
    and stops at comdgb_attach, or at comdgb_read_clsman given a structure
    file, through the snippets' simulationAbort (there is no CPU fallback).
    Skipped where the reference sources are absent."""
    from oracle.oracle import reference_dir
    ref = reference_dir()
    if ref is None:
        pytest.skip("reference sources not present on this machine")
    build()
    flat = os.path.join(ref, "src-flat")
    srcs = ["pmd.c", "docompute.c", "cmdLineParser.c", "domains.c", "eam.c", "ljForce.c",
            "ic_fcc.c", "cheby.c", "mycommand.c", "read.c", "write.c", "utility.c",
            "timestep.c"]
    for name in srcs:
        (tmp_path / name).write_text(open(os.path.join(flat, name)).read())
    includes, attach, read = _integration_snippets()
    assert '#include "comdgb.h"' in includes and "comdgb_attach(sim, &o)" in attach
    assert "comdgb_read_clsman(" in read
    d = (tmp_path / "docompute.c").read_text()
    d = _edit(d, '#include "read.h"\n', '#include "read.h"\n' + includes)
    d = _edit(d, '    printf("Initialization finished\\n");',
              "    {\n" + attach + "    }\n    printf(\"Initialization finished\\n\");")
    d = _edit(d, "eone = nTimeSteps(nsteps,data->sim,dt);",
              "eone = comdgb_nTimeSteps(nsteps, data->sim, dt);")
    d = _edit(d, "        sim = fromFileASCII(cmd, pot);", "        {\n" + read + "        }")
    (tmp_path / "docompute.c").write_text(d)
    p = (tmp_path / "pmd.c").read_text()
    p = _edit(p, '#include "pmd.h"\n', '#include "pmd.h"\n#include "comdgb.h"\n')
    p = _edit(p, "    destroySimulation(&sim);",
              "    comdgb_detach(sim);\n    destroySimulation(&sim);")
    (tmp_path / "pmd.c").write_text(p)
    lib = os.path.dirname(OUT)
    exe = tmp_path / "comd_dropin"
    flags = ["-O1", "-DDOUBLE", "-DUSE_CHEBY", "-DGZIPSUPPORT", "-I",
             os.path.join(flat, "include"), "-I", INCLUDE]
    objs = []
    for name in srcs:
        # the edited files: the library's types must be the reference's, and
        # every library call declared (pmd.c calls do_compute_work
        # undeclared in the reference itself)
        strict = {"docompute.c": ["-Werror=incompatible-pointer-types",
                                  "-Werror=implicit-function-declaration"],
                  "pmd.c": ["-Werror=incompatible-pointer-types"]}.get(name, ["-w"])
        obj = str(tmp_path / (name[:-2] + ".o"))
        r = subprocess.run(["gcc"] + flags + strict +
                           ["-c", str(tmp_path / name), "-o", obj], capture_output=True, text=True)
        assert r.returncode == 0, (name, r.stderr)
        objs.append(obj)
    r = subprocess.run(["gcc"] + objs + ["-o", str(exe), "-L", lib, "-lcomdgb",
                                         "-Wl,-rpath," + lib, "-lz", "-lm"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe), "-e", "-p", "cu", "-d", cg.POT_DIR, "-x", "4", "-y", "4",
                        "-z", "4"], capture_output=True, text=True, timeout=300,
                       env=dict(os.environ, CUDA_VISIBLE_DEVICES=""))
    assert r.returncode != 0
    assert "total atoms is: 256" in r.stdout, r.stdout[-2000:]
    assert "Error code: -30" in r.stderr, r.stderr[-2000:]  # the snippet's abort
    assert "Starting simulation" not in r.stdout
    # a structure file: the reader bins on GPU 0, so without one it fails
    r = subprocess.run([str(exe), "-e", "-p", "ag", "-d", cg.POT_DIR, "-f",
                        os.path.join(cg.DATA_DIR, "8k.inp.gz")], capture_output=True, text=True,
                       timeout=300, env=dict(os.environ, CUDA_VISIBLE_DEVICES=""))
    assert r.returncode != 0
    assert "Error code: -3\n" in r.stderr, r.stderr[-2000:]
    assert "Initialization finished" not in r.stdout
