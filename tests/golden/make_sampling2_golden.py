"""Golden trajectories of the reference's multi-state sampler (sampling2.sample).

Run here, where the reference source is mounted read-only:

    python tests/golden/make_sampling2_golden.py /root/reference/src

It imports the reference with the shims of ``make_golden.py`` plus one for
``sampling2.__transition_states``: that function calls
``numpy.searchsorted(..., side='leff')``, which numpy 2 rejects and older
numpy read by its first letter, so the shim maps 'leff' to 'left'.  Writes
``sampling2_goldens.npz`` next to this file.
"""

import os
import sys

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import import_reference  # noqa: E402


def main():
    src = sys.argv[1] if len(sys.argv) > 1 else "/root/reference/src"
    scopyon = import_reference(src)
    search = numpy.searchsorted

    def searchsorted(a, v, side="left", sorter=None):
        return search(a, v, side="left" if side == "leff" else side, sorter=sorter)

    numpy.searchsorted = searchsorted
    out = {}
    # two-dimensional, three states with transitions, periodic walls
    t = numpy.arange(9) * 1e-3
    pts = scopyon.sampling2.sample(
        t, N=[5, 3, 2], lower=-2e-6, upper=2e-6, D=[4e-13, 1e-13, 0.0],
        transmat=[[0.0, 150.0, 0.0], [120.0, 0.0, 30.0], [0.0, 200.0, 0.0]], ndim=2,
        periodic=True, rng=numpy.random.RandomState(3))
    out["s2a_t"] = t
    out["s2a_pts"] = numpy.array(pts)
    # three dimensions, one state, no transitions, no walls; a repeated time point
    t = numpy.array([0.0, 0.5e-3, 0.5e-3, 1.5e-3, 2.0e-3])
    pts = scopyon.sampling2.sample(
        t, N=4, lower=[-1e-6, -2e-6, -0.5e-6], upper=[1e-6, 2e-6, 0.5e-6], D=0.2e-12, ndim=3,
        rng=numpy.random.RandomState(8))
    out["s2b_t"] = t
    out["s2b_pts"] = numpy.array(pts)
    # two states, fast switching, periodic, 3-D with a flat z axis (lower == upper)
    t = numpy.arange(13) * 0.5e-3
    pts = scopyon.sampling2.sample(
        t, N=[30, 20], lower=[-3e-6, -3e-6, 0.0], upper=[3e-6, 3e-6, 0.0], D=[1e-12, 5e-14],
        transmat=[[0.0, 800.0], [600.0, 0.0]], ndim=3, periodic=True,
        rng=numpy.random.RandomState(21))
    out["s2c_t"] = t
    out["s2c_pts"] = numpy.array(pts)
    numpy.savez_compressed(os.path.join(HERE, "sampling2_goldens.npz"), **out)
    print("wrote", os.path.join(HERE, "sampling2_goldens.npz"))


if __name__ == "__main__":
    main()
