"""Drop-in check with pyMOTO itself (CPU): when pyMOTO is importable, this package's modules subclass
pymoto.Module and run inside pyMOTO's own Network, next to pyMOTO's modules, under pyMOTO's and this package's
finite_difference.  Runs in a subprocess where pyMOTO's sources are importable (the location the golden
fixtures were generated from); skipped where they are not."""
import os
import subprocess
import sys
import textwrap

import pytest

from conftest import GOLDEN, ROOT

sys.path.insert(0, GOLDEN)
import make_golden  # noqa: E402

pytestmark = pytest.mark.skipif(not make_golden.REF or not os.path.isdir(os.path.join(make_golden.REF, "pymoto")),
                                reason="pyMOTO's sources are not available here")

SCRIPT = textwrap.dedent('''
    import sys, os, numpy as np
    sys.path.insert(0, os.path.join(sys.argv[1], "tests", "golden"))
    import make_golden
    pym = make_golden.import_reference()
    import pymoto_gb300 as pg
    assert pg.HOST_RUNTIME == "pymoto", pg.HOST_RUNTIME
    assert issubclass(pg.Scaling, pym.Module) and issubclass(pg.ScalarToFile, pym.Module)
    np.random.seed(0)
    sx = pym.Signal("x", np.random.rand(12) + 0.2)
    with pym.Network() as fn:
        sv = pym.EinSum("i->")(sx)                                   # pyMOTO's module
        sg = pg.Scaling(scaling=5.0, maxval=3.0)(sv)                 # this package's module
        so = pg.Scaling(scaling=100.0)(sv)
        sv.tag, sg.tag = "volume", "constraint"
        log = pg.ScalarToFile(os.path.join(sys.argv[2], "log.txt"))
        log(sv, sg)
    fn.response()
    assert abs(sg.state - 5.0 * (sx.state.sum() - 3.0) / 3.0) < 1e-12
    def check(x0, dx, an, fd):
        assert abs(an - fd) <= 1e-6 * max(abs(an), 1e-12), (an, fd)
    pym.finite_difference(sx, [sg, so], fn, test_fn=check, verbose=False)   # pyMOTO's checker
    out = pg.finite_difference(sx, [sg, so], fn, dx=1e-6, verbose=False)   # this package's, on pyMOTO's network
    assert out == {"x": (0, 24)}, out
    log.flush()
    rows = open(os.path.join(sys.argv[2], "log.txt")).read().splitlines()
    assert rows[0].split("\\t") == ["Iteration", "volume", "constraint"], rows[0]
    assert len(rows) > 2 and rows[1].startswith("0\\t"), rows[:3]
    print("interop ok", len(rows))
''')


def test_modules_run_inside_a_pymoto_network(tmp_path):
    env = dict(os.environ, PYTHONPATH=ROOT, PYMOTO_GB300_STANDALONE="0")
    res = subprocess.run([sys.executable, "-c", SCRIPT, ROOT, str(tmp_path)], capture_output=True, text=True,
                         env=env, timeout=600)
    assert res.returncode == 0, res.stdout[-2000:] + res.stderr[-3000:]
    assert "interop ok" in res.stdout
