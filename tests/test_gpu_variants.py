"""The measurement switches change how the kernels work, never the results.

D4E_COMPACT=ld compacts with per-thread loads instead of the shared-memory
bulk-copy ring, D4E_STAGE_PLC=0 reads a single puzzle's placement table
through L1 instead of staging it in shared memory, and D4E_U32=0 keeps the
walk's copy counters in 64-bit words.  Each is read once per
process, so each runs in a child process over golden cases (single puzzle
and batch) whose counts must equal the reference's.
"""
import json
import os
import subprocess
import sys

import pytest

from conftest import REPO

pytestmark = pytest.mark.gpu

CHILD = r"""
import json, sys
sys.path.insert(0, sys.argv[1] + "/d4-pieces_gb300"); sys.path.insert(0, sys.argv[1])
from d4gb import engine as E
from d4gb.problem import Problem
cases = json.load(open(sys.argv[1] + "/tests/golden/cases.json"))["cases"][:12]
probs = [Problem(c["width"], c["height"], c["rows"], c["shapes"], c["counts"], c["sym"])
         for c in cases]
single = []
for p in probs:
    f = E.Frow(p.shapes, p.counts, p.sym, p.width, device=0)
    s = E.CudaSearcher(f, rows=p.rows)
    s.run()
    single.append(s.count())
batch = [r["count"] for r in E.batch_run(probs)[0]]
wide = [r["count"] for r in E.batch_run(probs, wide_keys=True)[0]]
print(json.dumps({"single": single, "batch": batch, "wide": wide,
                  "want": [c["count"] for c in cases]}))
"""


@pytest.mark.parametrize("env", [{"D4E_COMPACT": "ld"}, {"D4E_STAGE_PLC": "0"}, {"D4E_U32": "0"}])
def test_switch_keeps_counts(env):
    out = subprocess.run([sys.executable, "-c", CHILD, str(REPO)], capture_output=True,
                         text=True, timeout=600, env={**os.environ, **env})
    assert out.returncode == 0, out.stderr[-2000:]
    r = json.loads(out.stdout.strip().splitlines()[-1])
    assert r["single"] == r["want"]
    assert r["batch"] == r["want"]
    assert r["wide"] == r["want"]
