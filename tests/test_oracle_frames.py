"""The vectorised FP64 frame oracle (oracle/frames.py) against the per-particle
oracle, which the reference's own frames pin.

* The four golden frames: the same expectation (1e-13 of the image maximum),
  the same ADC counts, true_data (rtol 1e-14) and bleaching states.
* Random records, many near and past the image edges, at several depth keys
  (including the key past the depth cutoff) and two pixel sizes: the same
  footprint sums as ``overlay_signal_sat`` per record, per pixel.
"""

import numpy
import pytest

import oracle as O
from oracle import frames as F
from golden_cases import (FRAME_CASES, case_bleach, case_frames_draws, case_inputs, case_params,
                          case_tree)


@pytest.mark.parametrize("name,nframes,tag", FRAME_CASES)
def test_fast_frames_match_per_particle_oracle(golden, name, nframes, tag):
    params = case_params(golden, name, tag)
    data = case_inputs(golden, name)
    frames = case_frames_draws(golden, name, nframes)
    if case_tree(golden, name)["default"]["detector"]["type"] == "CMOS":
        for d in frames:
            d["noise"] = O.cmos_table_draw(golden["cmos_table"], d["uniform"])
    bleach = case_bleach(golden, name)
    bleaching = params.bleach_switch and name != "fa"  # form_image keeps no states
    s1 = {} if bleaching else None
    s2 = {} if bleaching else None
    d1, d2 = O.InjectedDraws(bleach, frames), O.InjectedDraws(bleach, frames)
    for f in range(nframes):
        c1, i1 = O.output_frame(params, data, d1, f, states=s1)
        c2, i2 = F.output_frame_fast(params, data, d2, f, states=s2)
        e_ref = golden["%s_expectation" % name][f]
        assert numpy.abs(c2[:, :, 0] - c1[:, :, 0]).max() <= 1e-13 * c1[:, :, 0].max()
        assert numpy.abs(c2[:, :, 0] - e_ref).max() <= 1e-13 * e_ref.max()
        numpy.testing.assert_array_equal(c2[:, :, 1], c1[:, :, 1])
        assert list(i2["true_data"]) == list(i1["true_data"])
        for m in i1["true_data"]:
            numpy.testing.assert_allclose(i2["true_data"][m], i1["true_data"][m], rtol=1e-14)
        if bleaching:
            assert i2["fluorescence_states"] == i1["fluorescence_states"]


@pytest.mark.parametrize("px,shape", [(160e-9, (40, 24)), (66e-9, (33, 50))])
def test_fast_splat_matches_overlay_sat(px, shape):
    rng = numpy.random.RandomState(17)
    geom = F.QuadrantGeometry()
    nw, nh = shape
    for depth in (0.0, 313e-9, 999.4e-9, 1.2e-6):
        key = int(F.depth_keys([depth])[0])
        depth_value = 1000e-9 if key < 0 else key * 1e-9
        psf_r = O.born_wolf_radial(geom.r, depth_value, 5.78e-7)
        n = 60
        # positions over the image and up to 1.5 um past its edges
        x = rng.uniform(-(nw * px / 2 + 1.5e-6), nw * px / 2 + 1.5e-6, n)
        y = rng.uniform(-(nh * px / 2 + 1.5e-6), nh * px / 2 + 1.5e-6, n)
        w = rng.uniform(0.5, 2.0, n)
        got = numpy.zeros(shape)
        F.splat_records(got, F.quadrant_prefix(geom, psf_r), geom.n, x, y, w, px)
        full = O.radial_to_cartesian(geom.r, psf_r)
        sat = numpy.zeros((full.shape[0] + 1, full.shape[1] + 1))
        sat[1:, 1:] = full.cumsum(0).cumsum(1)
        ref = numpy.zeros(shape)
        for k in range(n):
            O.overlay_signal_sat(ref, sat, [0.0, x[k], y[k]], px, w[k])
        assert numpy.abs(got - ref).max() <= 1e-12 * ref.max()
        assert numpy.array_equal(got > 0, ref > 0)


def test_depth_keys_match_scalar_rule():
    d = numpy.array([0.0, -0.4e-9, 1e-9, -999.9e-9, 1000.5e-9, 1001e-9, 3e-6, -2e-6])
    numpy.testing.assert_array_equal(F.depth_keys(d), [O.psf_depth_key(v)[0] for v in d])
