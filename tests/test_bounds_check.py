"""The bounds-checked build (-DPN_BOUNDS_CHECK, libpn_gb300_bc.so): every device index of
the build and of the traversals is checked before it reaches memory, the first failure
going to the search's error word (site and index, pn_bounds_failure).  The parity suite's
2D and 3D clouds (bounds_check_cases.py) run through both libraries in child processes:
the checked run reports no failure, and every output equals the normal build's bit for bit
(the checks only read indices)."""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(lib, out):
    env = dict(os.environ, PN_GB300_LIB=lib)
    r = subprocess.run([sys.executable, os.path.join(ROOT, "tests", "bounds_check_cases.py"),
                        out], env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-4000:]
    return np.load(out)


def test_bounds_checked_build_matches(tmp_path):
    import __graft_entry__
    __graft_entry__.build()
    pn_build = __graft_entry__.package().build  # the package's build script
    lib = pn_build.build()
    lib_bc = pn_build.build(bounds_check=True)
    plain = _run(lib, str(tmp_path / "plain.npz"))
    checked = _run(lib_bc, str(tmp_path / "checked.npz"))
    assert int(plain["build_flags"][0]) == 0 and int(checked["build_flags"][0]) == 1
    names = list(checked["status_names"])
    for name, (err, site, index) in zip(names, checked["status"]):
        assert (err, site) == (0, 0), f"{name}: status {err}, bounds site {site} index {index}"
    assert int(checked["incremental/n_overflow"][0]) > 0  # the overflow lists were walked
    keys = [k for k in plain.files if k not in ("build_flags", "status", "status_names")]
    assert set(keys) == {k for k in checked.files
                         if k not in ("build_flags", "status", "status_names")}
    for k in keys:
        assert np.array_equal(plain[k], checked[k]), k
