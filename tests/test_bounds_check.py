"""The bounds-checked build (every gathered index tested against its array,
the stand-in for compute-sanitizer) runs the passes without a violation and
gives the same results as the normal build."""

import os
import subprocess
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_normal_build_reports_no_checking(gmvs_lib):
    assert gmvs_lib.gmvs_bounds_violations(0) == -1


@pytest.mark.gpu
def test_checked_build_no_violations_same_results(gmvs_lib, cuda, tmp_path):
    from gmvs_gb300 import build

    lib = build.build(defines=("GMVS_BOUNDS_CHECK=1",), out_dir=str(tmp_path / "checked"))
    outs = {}
    for name, path in (("checked", lib), ("normal", build.LIB_PATH)):
        dst = str(tmp_path / f"{name}.npz")
        env = dict(os.environ, GMVS_GB300_LIB=os.path.abspath(path),
                   PYTHONPATH=os.pathsep.join([HERE, os.path.dirname(HERE), os.environ.get("PYTHONPATH", "")]))
        r = subprocess.run([sys.executable, os.path.join(HERE, "bounds_case.py"), dst], env=env,
                           capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        outs[name] = dict(np.load(dst))
    assert int(outs["checked"]["violations"]) == 0
    assert int(outs["normal"]["violations"]) == -1
    for k, v in outs["normal"].items():
        if k != "violations":
            assert np.array_equal(outs["checked"][k], v, equal_nan=True), k
