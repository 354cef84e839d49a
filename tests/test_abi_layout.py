"""The drop-in boundary's data model is the reference's, member for member.

include/comdgb_simflat.h restates the -DDOUBLE structs of the reference
(simflat_t src-flat/include/pmdTypes.h:104-141, pmd_base_potential_t
:74-79, potentialarray_t src-flat/include/eamTypes.h:68-74, eampotential_t
:92-101, eam_cheby_t :104-114, ljpotential_t src-flat/include/ljTypes.h:
72-81), so that a host built by the reference's own setup code can hand its
pointers to the library.  This test compiles a probe against the
reference's headers (-DDOUBLE) that prints sizeof and offsetof of every
member, then compiles a second translation unit against the library's
header whose _Static_asserts must hold for those numbers.  CPU only; it
needs the reference sources and is skipped where they are absent.
"""
import os
import subprocess

import pytest

from oracle.oracle import reference_dir

# struct -> members, as declared in include/comdgb_simflat.h
MEMBERS = {
    "simflat_t": ["stateflag", "nbx", "nboxes", "ntot", "bounds", "boxsize", "dcenter", "natoms",
                  "id", "iType", "mass", "r", "p", "f", "rho", "fi", "e", "nAtoms", "pot",
                  "comment", "stress", "defgrad", "bf", "ch_pot"],
    "pmd_base_potential_t": ["cutoff", "mass", "force", "destroy"],
    "potentialarray_t": ["n", "x0", "xn", "invDx", "values"],
    "eampotential_t": ["cutoff", "mass", "force", "destroy", "phi", "rho", "f", "lat"],
    "eam_cheby_t": ["cutoff", "mass", "phi", "rho", "f", "dphi", "drho", "df", "lat"],
    "ljpotential_t": ["cutoff", "mass", "force", "destroy", "sigma", "epsilon"],
}

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _probe_source():
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "pmdTypes.h"',
             '#include "ljTypes.h"',
             # memUtils.h's inline allocators name two of the reference's
             # functions; the probe never calls them
             "void breakinme() {}", "int suAbort(int status, char *msg) { (void)msg; return status; }",
             "int main(void) {"]
    for st, mem in MEMBERS.items():
        lines.append(f'  printf("{st} sizeof %zu\\n", sizeof({st}));')
        for m in mem:
            lines.append(f'  printf("{st} {m} %zu %zu\\n", offsetof({st}, {m}), '
                         f'sizeof((({st} *)0)->{m}));')
    lines += ["  return 0;", "}"]
    return "\n".join(lines) + "\n"


def test_simflat_layout_matches_reference_headers(tmp_path):
    ref = reference_dir()
    if ref is None:
        pytest.skip("reference sources not present on this machine")
    probe = tmp_path / "probe.c"
    probe.write_text(_probe_source())
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-DDOUBLE", "-I", os.path.join(ref, "src-flat", "include"),
                    str(probe), "-o", str(exe)], check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    asserts = ["#include <stddef.h>", '#include "comdgb_simflat.h"']
    n = 0
    for line in out.splitlines():
        f = line.split()
        if f[1] == "sizeof":
            asserts.append(f'_Static_assert(sizeof({f[0]}) == {f[2]}, "sizeof {f[0]}");')
        else:
            asserts.append(f'_Static_assert(offsetof({f[0]}, {f[1]}) == {f[2]}, '
                           f'"offsetof {f[0]}.{f[1]}");')
            asserts.append(f'_Static_assert(sizeof((({f[0]} *)0)->{f[1]}) == {f[3]}, '
                           f'"sizeof {f[0]}.{f[1]}");')
        n += 1
    assert n == sum(len(m) + 1 for m in MEMBERS.values())
    check = tmp_path / "layout_check.c"
    check.write_text("\n".join(asserts) + "\n")
    r = subprocess.run(["gcc", "-std=c11", "-c", "-I", os.path.join(ROOT, "include"), str(check),
                        "-o", str(tmp_path / "layout_check.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_python_binding_structs_match_the_library_header(tmp_path):
    """The ctypes mirrors the tests and bench.py pass through the C ABI
    (comd_gb300/abi.py, comd_gb300/lib.py) have the sizes and member offsets
    of include/comdgb.h, as the host compiler lays the structs out."""
    import ctypes as C

    from comd_gb300 import abi
    from comd_gb300.lib import Opts, Tune
    mirrors = {"simflat_t": abi.SimFlat, "pmd_base_potential_t": abi.BasePotential,
               "potentialarray_t": abi.PotentialArray, "eampotential_t": abi.EamPotential,
               "eam_cheby_t": abi.EamCheby, "ljpotential_t": abi.LjPotential,
               "comdgb_opts": Opts, "comdgb_tune": Tune}
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "comdgb.h"',
             "int main(void) {"]
    for st, py in mirrors.items():
        lines.append(f'  printf("{st} sizeof %zu\\n", sizeof({st}));')
        for name, _ in py._fields_:
            lines.append(f'  printf("{st} {name} %zu\\n", offsetof({st}, {name}));')
    lines += ["  return 0;", "}"]
    probe = tmp_path / "probe.c"
    probe.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(probe), "-o",
                    str(exe)], check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    seen = 0
    for line in out.splitlines():
        st, name, val = line.split()
        py = mirrors[st]
        got = C.sizeof(py) if name == "sizeof" else getattr(py, name).offset
        assert got == int(val), (st, name, got, val)
        seen += 1
    assert seen == sum(len(p._fields_) + 1 for p in mirrors.values())


def test_public_headers_compile_cleanly_as_c99_and_cxx11(tmp_path):
    """include/*.h compile without a warning in a C99 and a C++11 caller
    (-pedantic -Wall -Wextra -Werror): the reference's host is C, and the
    headers carry their own extern "C" guards"""
    src = '#include "comdgb.h"\n#include "comdgb_seed.h"\nint main(void) { return 0; }\n'
    for compiler, std, ext in (("gcc", "-std=c99", "c"), ("g++", "-std=c++11", "cpp")):
        f = tmp_path / f"hdr.{ext}"
        f.write_text(src)
        r = subprocess.run([compiler, std, "-pedantic", "-Wall", "-Wextra", "-Werror", "-I",
                            os.path.join(ROOT, "include"), "-c", str(f), "-o",
                            str(tmp_path / f"hdr_{ext}.o")], capture_output=True, text=True)
        assert r.returncode == 0, (compiler, r.stderr)


def test_integration_batch_and_gradient_example_compiles(tmp_path):
    """The C example of INTEGRATION.md's "Batches and gradients" section
    compiles against include/comdgb.h as written (inside a function that
    declares the handles and inputs it names), so the document keeps up
    with the header"""
    import re
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    sec = text.split("## Batches and gradients", 1)[1]
    code = re.search(r"```c\n(.*?)```", sec, re.S).group(1)
    src = ("#include <stddef.h>\n#include \"comdgb.h\"\n"
           "void example(comdgb_opts o, comdgb_sim *h, const double *target_forces_by_id) {\n"
           + code + "\n}\n")
    f = tmp_path / "example.c"
    f.write_text(src)
    # (the example leaves reps[] to the caller's set-up: no use-before-set
    # warnings)
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wno-unused-variable", "-Wno-uninitialized",
                        "-Wno-maybe-uninitialized", "-Werror", "-I",
                        os.path.join(ROOT, "include"), "-c", str(f), "-o",
                        str(tmp_path / "example.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_integration_python_example_runs_to_the_gpu_boundary():
    """INTEGRATION.md's ctypes example, run as written without a GPU: every
    name it uses exists, the attach returns the library's CUDA error and
    nTimeSteps on the unattached simulation returns NaN (no CPU fallback)"""
    import re
    import sys
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    sec = text.split("## Python (ctypes) binding", 1)[1]
    code = re.search(r"```python\n(.*?)```", sec, re.S).group(1)
    code += ("\nimport math\nassert L.comdgb_last_error(None, 0) >= 0\n"
             "print('E', e, math.isnan(e))\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True,
                       timeout=300, env=dict(os.environ, CUDA_VISIBLE_DEVICES="",
                                             PYTHONPATH=ROOT))
    assert r.returncode == 0, r.stderr[-2000:]
    assert "E nan True" in r.stdout, r.stdout
