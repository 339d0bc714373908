"""GPU: the reference's own sor1 example, recompiled against the drop-in.

oracle/_ref/sor1_dropin is the reference's examples/sor1 (main.cpp,
Solver.cpp, Timing.cpp and the Utils mesh code), unmodified, compiled
against this project's source-compatible headers (include/bcmtools:
BlockManager, Scalar3D, Scalar3DUpdater ahead of the reference's include/)
and linked to libbcmg.so, so that its BlockManager::beginUpdateVC /
endUpdateVC run the ghost update on the GPU while its own sweep stays on the
host.  Run on the example's shipped configuration it must print the
reference's one known answer, errorMax = 0.00353051 (examples/sor1/log.4:54),
in both of its VC-update modes (all faces at once, and per axis).
"""
import os
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

BIN = Path(__file__).resolve().parents[1] / "oracle" / "_ref" / "sor1_dropin"

# examples/sor1/test.conf: simple tree of levels 0..3, random leaf order,
# fixed values on the x faces (periodic y and z), 400 outer x 1 inner SOR
# iterations at omega 1.2, 2^3 cells per block, one virtual cell.
CONF = """minLevel = 0
maxLevel = 3
treeType = simple
ordering = random
type = x
nLoopOuter = 400
nLoopInner = 1
omega = 1.2
size = 2
vc = 1
output = out.dat
"""


@pytest.mark.parametrize("separate", [False, True])
def test_reference_sor1_recompiled_against_dropin(gpu_ok, tmp_path, separate):
    if not BIN.exists():
        pytest.skip("oracle/_ref/sor1_dropin not built (needs the reference's expanded sources)")
    conf = tmp_path / "test.conf"
    conf.write_text(CONF + ("separateVCUpdate = true\n" if separate else ""))
    env = dict(os.environ, OMP_NUM_THREADS="1", BCMG_DEVICE="0")
    r = subprocess.run([str(BIN), str(conf)], cwd=tmp_path, capture_output=True, text=True,
                       timeout=300, env=env)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("errorMax = ")]
    assert lines == ["errorMax = 0.00353051"], r.stdout[-2000:]
    # the layout report of the drop-in BlockManager: 456 blocks on one rank
    assert "    total: 456" in r.stdout
