"""The oracle against golden vectors recorded from the reference scopyon.

Every test here runs on the CPU.  Tolerances: PSF and footprint sums within a
few FP64 ulps of the reference; ADC counts, bleaching budgets and
``true_data`` bit-exact; EMCCD and CMOS draws exact.
"""

import numpy
import pytest

import oracle as O
from golden_cases import (FRAME_CASES, case_bleach, case_frames_draws, case_inputs,
                          case_params, case_tree)

R = O.radial_grid()


@pytest.mark.parametrize("name,wl", [("tritc", 5.78e-7), ("egfp", 5.08e-7)])
def test_born_wolf_radial_and_depth_keys(golden, name, wl):
    for i, d in enumerate(golden["psf_depths"]):
        key, dv = O.psf_depth_key(d)
        assert key == golden["psf_%s_keys" % name][i]
        ref = golden["psf_%s_radial" % name][i]
        mine = O.born_wolf_radial(R, dv, wl)
        assert numpy.abs(mine - ref).max() <= 2e-15 * ref.max()


def test_gaussian_radial(golden):
    numpy.testing.assert_array_equal(O.gaussian_radial(R, 1e-7), golden["psf_gauss100_radial"])


def test_cartesian_grid(golden):
    cart = O.radial_to_cartesian(R, golden["psf_tritc_radial"][0])
    idx = tuple(golden["cart_samples_idx"].T)
    numpy.testing.assert_array_equal(cart[idx], golden["cart_samples"])
    assert abs(cart.sum() - golden["cart_total"]) <= 1e-12 * golden["cart_total"]


@pytest.mark.parametrize("depth_idx", [0, 3])
@pytest.mark.parametrize("case", ["c40_px160", "c96x64_px66"])
def test_overlay_exact_and_sat(golden, case, depth_idx):
    radial = golden["psf_tritc_radial"][depth_idx]
    tab = O.radial_to_cartesian(R, radial)
    sat = numpy.zeros((2000, 2000))
    sat[1:, 1:] = tab.cumsum(0).cumsum(1)
    px = float(golden["ov_%s_px" % case])
    for p, ref in zip(golden["ov_%s_pos" % case], golden["ov_%s_d%d" % (case, depth_idx)]):
        exact = numpy.zeros(ref.shape)
        O.overlay_signal(exact, tab, [0.0, p[0], p[1]], px, 1.0)
        numpy.testing.assert_allclose(exact, ref, rtol=1e-13, atol=0)
        viasat = numpy.zeros(ref.shape)
        O.overlay_signal_sat(viasat, sat, [0.0, p[0], p[1]], px, 1.0)
        nz = ref > 0
        assert numpy.array_equal(viasat > 0, nz)
        if nz.any():
            assert (numpy.abs(viasat - ref)[nz] / ref[nz]).max() < 1e-8


def test_overlay_small_pixels_512(golden):
    cart = O.radial_to_cartesian(R, golden["psf_tritc_radial"][0])
    img = numpy.zeros((512, 512))
    O.overlay_signal(img, cart, numpy.zeros(3), 4.444444444444444e-08, 1.0)
    i0, i1, j0, j1 = golden["ov_512_px44_window"]
    numpy.testing.assert_allclose(img[i0:i1, j0:j1], golden["ov_512_px44"], rtol=1e-13)
    assert img.sum() == pytest.approx(img[i0:i1, j0:j1].sum(), rel=1e-15)


def test_quadrant_sat_reproduces_full_grid_sums(golden):
    radial = golden["psf_tritc_radial"][3]
    quad = O.quadrant_sat(R, radial)
    full = O.radial_to_cartesian(R, radial)
    # the quadrant table is the lower-right quarter of the full grid
    numpy.testing.assert_allclose(quad[1:, 1:][-1, -1], full[999:, 999:].sum(), rtol=1e-13)
    numpy.testing.assert_allclose(quad[1:, 1:][0, 0], full[999, 999], rtol=0)


def test_physics(golden):
    for angle, amp, pen, n1, n2 in golden["physics_rows"]:
        a, p = O.snells_law(400000.0, 532e-9, angle)
        assert a == amp and p == pen
        assert O.emit_photons(a, 1.0, 83400, 0.61, 20e-9) == n1
        assert O.emit_photons(a * 0.37, 3e-3, 56000, 0.6, 2.0e-9) == n2


def test_emccd_distribution_and_draws(golden):
    for e in (0.01, 0.5, 1.0, 3.7, 10.0, 55.0, 100.0, 333.3, 700.0):
        s_ref, p_ref = golden["emccd_pdf_%g" % e]
        s, p = O.emccd_distribution(e, 300)
        numpy.testing.assert_array_equal(s, s_ref)
        numpy.testing.assert_allclose(p, p_ref, rtol=1e-12, atol=1e-300)
    for e, g, u, sig in golden["emccd_draws"]:
        assert O.emccd_draw(e, int(g), u) == sig


def test_emccd_beyond_reference_overflow():
    # the reference raises "probabilities contain NaN" above ~709 e-; the
    # shifted restatement keeps a proper distribution with mean ~ g * E
    s, p = O.emccd_distribution(1200.0, 300)
    assert numpy.isfinite(p).all() and abs(p.sum() - 1) < 1e-12
    mean = (s * p).sum()
    assert abs(mean / (300 * 1200.0) - 1) < 0.01


@pytest.mark.parametrize("fpn", ["none", "pixel", "column"])
def test_adc_maps(golden, fpn):
    class Fixed:
        def normal(self, *a, **k):
            return golden["adc_%s_normals" % fpn]

    count = {"none": 0.0, "pixel": 5.0, "column": 3.0}[fpn]
    off, gain = O.adc_maps(6, 5, 12, 800000, 100, fpn, count, Fixed())
    numpy.testing.assert_array_equal(off, golden["adc_%s_offset" % fpn])
    numpy.testing.assert_array_equal(gain, golden["adc_%s_gain" % fpn])


def test_sample_inputs(golden):
    t = numpy.arange(7) * 0.5e-3
    out = O.sample_inputs(t, 5, [-1e-6, -2e-6, -0.5e-6], [1e-6, 2e-6, 0.5e-6], 0.1e-12, 3,
                          numpy.random.RandomState(5))
    numpy.testing.assert_array_equal(numpy.array([p for _, p in out]), golden["samp3_pts"])
    numpy.testing.assert_array_equal(numpy.array([x for x, _ in out]), golden["samp3_t"])
    out = O.sample_inputs(t[:4], 4, -3e-6, 3e-6, [0.2e-12, 0.05e-12], 2,
                          numpy.random.RandomState(9))
    numpy.testing.assert_array_equal(numpy.array([p for _, p in out]), golden["samp2_pts"])


@pytest.mark.parametrize("name,nframes,tag", FRAME_CASES)
def test_frames_injected(golden, name, nframes, tag):
    params = case_params(golden, name, tag)
    data = case_inputs(golden, name)
    frames = case_frames_draws(golden, name, nframes)
    if case_tree(golden, name)["default"]["detector"]["type"] == "CMOS":
        for d in frames:
            d["noise"] = O.cmos_table_draw(golden["cmos_table"], d["uniform"])
    draws = O.InjectedDraws(case_bleach(golden, name), frames)
    ids = [int(i) for i in golden["%s_true_ids" % name]]
    if name == "fa":
        results = [O.output_frame(params, data, draws)]
    else:
        results = O.generate_frames(params, data, nframes, draws, use_sat=(name == "fd"))
    for f, (cam, info) in enumerate(results):
        e_ref = golden["%s_expectation" % name][f]
        assert numpy.abs(cam[:, :, 0] - e_ref).max() <= 1e-13 * e_ref.max()
        numpy.testing.assert_array_equal(cam[:, :, 1], golden["%s_adc" % name][f])
        td = numpy.array([info["true_data"][m] for m in ids])
        numpy.testing.assert_allclose(td, golden["%s_true_data" % name][f], rtol=1e-14)
        if "%s_states" % name in golden:
            st = numpy.array([info["fluorescence_states"][m] for m in ids])
            numpy.testing.assert_array_equal(st, golden["%s_states" % name][f])


def test_frames_numpy_rng_matches_reference_stream(golden):
    # the oracle, fed the same seeded RandomState, makes the same draws as the reference
    params = case_params(golden, "fa", "egfp")
    cam, _ = O.output_frame(params, case_inputs(golden, "fa"),
                            O.NumpyDraws(numpy.random.RandomState(7)))
    numpy.testing.assert_array_equal(cam[:, :, 1], golden["fa_adc"][0])
