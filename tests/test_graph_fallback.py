"""The step graphs with and without conditional nodes give the same state bit
for bit.  In force order a step's rebuild section (classification, rebin,
compaction, list build) and the refresh of the slot-order FP32 copy after a
list overflow are conditional graph nodes; with COMDGB_GRAPH_CONDITIONALS=0
(read once per process: how kernel-level profiles are taken, since ncu
profiles no kernel of a graph with a conditional node) the same kernels are
launched in every step and stand down by themselves.  Each run is a child
process; both hash the state after 40 steps with list rebuilds."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import hashlib, sys
sys.path.insert(0, sys.argv[1])
import numpy as np
import comd_gb300 as cg
from comd_gb300.abi import by_id
pot = cg.eam_potential("cu")
s = cg.fcc(10, 10, 10, pot.ptr.contents.lat, 1.0, 1.0, pot)
cg.seed(s, 7, cg.DISP_GAUSSIAN, 0.05, 1200.0, pot.ptr.contents.mass)
d = cg.DeviceSim(s, cg.opts(cg.POT_EAM_CHEBY, cg.PREC_MIXED, skin=0.2))
assert d.list_info()[0]
e, _ = d.steps(40, 1e-15)
builds = d.list_info()[2]
d.download(s)
d.close()
h = hashlib.sha256()
for f in ("r", "p", "f"):
    h.update(np.ascontiguousarray(by_id(s, f)).tobytes())
print(builds, repr(e), h.hexdigest())
"""


def run(conditionals):
    env = dict(os.environ)
    env["COMDGB_GRAPH_CONDITIONALS"] = "1" if conditionals else "0"
    out = subprocess.run([sys.executable, "-c", CHILD, ROOT], env=env, capture_output=True,
                         text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    return out.stdout.strip().splitlines()[-1].split()


def test_conditional_nodes_do_not_change_the_trajectory():
    with_nodes = run(True)
    inline = run(False)
    assert int(with_nodes[0]) >= 2, with_nodes  # the rebuild section ran
    assert with_nodes == inline
