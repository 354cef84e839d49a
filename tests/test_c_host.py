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
from comd_gb300.build import HOST_OUT, build
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
