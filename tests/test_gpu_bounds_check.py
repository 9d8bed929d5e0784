"""GPU: the bounds-checked build (-DSC_BOUNDS_CHECK).

The library built with the flag range-checks the kernels' data-dependent
indices (a splat warp's tile buffer and block-copy ring, the register
splat's tile buffer, the tile buffers a pixel's merge reads, a record's bin
and its place in the bin lists), skips an access out of range and reports
it in the status words (bit 8).  Frames of the device and host paths and a
cursor binning, run in child processes with the normal and the checked
library, give the same arrays bit for bit, and no check fires (any status
bit raises in the child).
"""

import os
import subprocess
import sys

import numpy
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_bounds_checked_build_gives_the_same_frames(tmp_path):
    from scopyon_gb300 import _build
    normal = _build.build()
    checked = _build.build_checked()
    assert checked != normal and os.path.exists(checked)
    outs = []
    for name, lib in (("normal", normal), ("checked", checked)):
        path = str(tmp_path / (name + ".npz"))
        env = dict(os.environ, SCOPYON_GB300_LIB=lib)
        proc = subprocess.run([sys.executable, os.path.join(HERE, "bounds_check_frames.py"), path],
                              env=env, capture_output=True, text=True, timeout=900)
        assert proc.returncode == 0, proc.stdout[-2000:] + proc.stderr[-4000:]
        outs.append(numpy.load(path))
    a, b = outs
    assert sorted(a.files) == sorted(b.files)
    for k in a.files:
        numpy.testing.assert_array_equal(a[k], b[k], err_msg=k)
    assert a["device_8_4_4"].max() > 0 and a["host"].std() > 0
