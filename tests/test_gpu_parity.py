"""GPU parity: the CUDA path against the reference goldens and the oracle.

Tolerances (stated per test):
* PSF radial tables: 1e-12 relative to the table maximum (FP64 on both sides).
* Quadrant summed-area tables: hi + lo within 4 * 2^-48 of the FP64 oracle.
* Expected photon images: <= 1e-5 relative per pixel for pixels above 1e-6
  of the image maximum, and 1e-6 norm-wise.
* ADC: exact up to FP64 rounding (1e-9 ADU), except EMCCD inverse-CDF draws
  where at most max(1, 1e-4 * pixels) pixels may differ, by at most 1 ADU.
"""

import ctypes
import json

import numpy
import pytest

import oracle as O
from golden_cases import FRAME_CASES, case_frames_draws, case_raw_inputs, case_tree

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from scopyon_gb300 import _build, _lib
    _build.build()
    return _lib


def _dev(a, dtype=torch.float64):
    return torch.as_tensor(numpy.ascontiguousarray(a), dtype=dtype, device="cuda")


@pytest.mark.parametrize("name,wl", [("tritc", 5.78e-7), ("egfp", 5.08e-7)])
def test_psf_radial_born_wolf(lib, golden, name, wl):
    keys = golden["psf_%s_keys" % name]
    depths = numpy.array([1000e-9 if k == -1 else k * 1e-9 for k in keys])
    out = torch.empty((len(depths), 1000), dtype=torch.float64, device="cuda")
    lib.call("sc_psf_radial", lib.PSF_BORN_WOLF, wl, 1.4, 0.0, lib.ptr(_dev(depths)), len(depths),
             1000, 1e-9, lib.ptr(out), lib.stream_ptr())
    ref = golden["psf_%s_radial" % name]
    got = out.cpu().numpy()
    for i in range(len(depths)):
        assert numpy.abs(got[i] - ref[i]).max() <= 1e-12 * ref[i].max()


def test_psf_radial_gaussian(lib, golden):
    out = torch.empty((2, 1000), dtype=torch.float64, device="cuda")
    lib.call("sc_psf_radial", lib.PSF_GAUSSIAN, 0.0, 0.0, 1.0e-7, None, 2, 1000, 1e-9,
             lib.ptr(out), lib.stream_ptr())
    ref = golden["psf_gauss100_radial"]
    numpy.testing.assert_allclose(out.cpu().numpy()[1], ref, rtol=1e-14, atol=0)


def test_quadrant_sat(lib, golden):
    radial = golden["psf_tritc_radial"][[0, 3]]
    pitch = 1004
    sat = torch.zeros(2 * 1001 * pitch * 2, dtype=torch.float32, device="cuda")
    lib.call("sc_psf_quadrant_sat", lib.ptr(_dev(radial)), 2, 1000, 1e-9, lib.ptr(sat), pitch,
             lib.stream_ptr())
    got = sat.cpu().numpy().reshape(2, 1001, pitch, 2).astype(numpy.float64)
    r = O.radial_grid()
    for k in range(2):
        ref = O.quadrant_sat(r, radial[k])
        val = got[k, :, :1001, 0] + got[k, :, :1001, 1]
        assert numpy.abs(val - ref).max() <= 4 * 2.0 ** -48 * ref.max()


def test_box_table(lib, golden):
    """Box-integrated entries against FP64 sums of the full cartesian grid."""
    radial = golden["psf_tritc_radial"][[3]]
    pitch, P = 1004, 160
    sat = torch.zeros(1001 * pitch * 2, dtype=torch.float32, device="cuda")
    lib.call("sc_psf_quadrant_sat", lib.ptr(_dev(radial)), 1, 1000, 1e-9, lib.ptr(sat), pitch,
             lib.stream_ptr())
    nq = (1999 + P - 1) // P + 1
    nb = lib.load().sc_box_block_floats(nq)
    assert nb >= nq * nq and nb % 4 == 0
    box = torch.full((P * P * nb,), -1.0, dtype=torch.float32, device="cuda")
    lib.call("sc_psf_box_table", lib.ptr(sat), 1, 1000, pitch, P, lib.ptr(box), lib.stream_ptr())
    blocks = box.cpu().numpy().reshape(P, P, nb)
    assert (blocks[:, :, nq * nq:] == 0).all()  # block padding
    got = blocks[:, :, :nq * nq].reshape(P, P, nq, nq)
    full = O.radial_to_cartesian(O.radial_grid(), radial[0])
    csum = numpy.zeros((2000, 2000))
    csum[1:, 1:] = full.cumsum(0).cumsum(1)
    rng = numpy.random.RandomState(0)
    for _ in range(400):
        rx, ry = rng.randint(P, size=2)
        qx, qy = rng.randint(nq, size=2)
        mx, my = qx * P + rx - P, qy * P + ry - P
        a0, a1 = max(mx, 0), min(mx + P, 1999)
        b0, b1 = max(my, 0), min(my + P, 1999)
        ref = 0.0 if a1 <= a0 or b1 <= b0 else (
            csum[a1, b1] - csum[a0, b1] - csum[a1, b0] + csum[a0, b0])
        v = got[rx, ry, qx, qy]
        assert abs(v - ref) <= 2e-7 * abs(ref) + 1e-9 * csum[-1, -1] * 1e-9, (rx, ry, qx, qy)


def _config_from_tree(tree, **gpu):
    import scopyon_gb300 as sg
    tree = json.loads(json.dumps(tree))
    tree["default"]["gpu"] = dict(gpu)
    return sg.Configuration(yaml=tree)


@pytest.mark.parametrize("box", [True, False])
@pytest.mark.parametrize("depth_idx", [0, 3])
@pytest.mark.parametrize("case", ["c40_px160", "c96x64_px66"])
def test_single_emitter_footprints(lib, golden, case, depth_idx, box):
    """One emitter per sub-step through steps -> bin -> splat, against overlay_signal_.

    box=True takes the box-table path where it applies (integer px, generic
    positions); box=False forces the summed-area path everywhere."""
    from scopyon_gb300.config import DefaultConfiguration
    from scopyon_gb300.epifm import EngineConfig, FramePipeline
    px = float(golden["ov_%s_px" % case])
    shape = golden["ov_%s_d%d" % (case, depth_idx)].shape[1:]
    cfg = DefaultConfiguration()
    cfg.update({"default": {
        "magnification": 1.0, "detector": {"pixel_length": px, "image_size": list(shape)},
        "effects": {"photo_bleaching": {"switch": False}},
        "gpu": {"psf_wavelength": 5.78e-07, "box_tables": box}}})
    eng = EngineConfig(cfg["default"])
    assert eng.px == px
    assert eng.box_p == (160 if (box and case == "c40_px160") else 0)
    pipe = FramePipeline(eng, "cuda")
    pipe.merge_camera = False  # keep the splat's photon image (pipe.image)
    depth = float(golden["psf_depths"][depth_idx])
    n_emit = eng.qy * (eng.amplitude0 * numpy.exp(-abs(depth) / eng.penetration) * eng.x_sec
                       * 1.0) * eng.beer
    pos = golden["ov_%s_pos" % case]
    parts = numpy.zeros((len(pos), 1, 5))
    parts[:, 0, 0] = depth
    parts[:, 0, 1:3] = pos
    parts[:, 0, 4] = 4.0 * numpy.pi / (eng.norm_coeff * n_emit)
    pipe.psf.ensure(eng.depth_keys(parts[:, 0, 0]))
    for s in range(len(pos)):
        pipe.run_frame(parts[s:s + 1], numpy.array([1.0]), with_optinfo=False,
                       bleaching=False, seed=1)
        img = pipe.image.cpu().numpy().astype(numpy.float64).reshape(shape)
        ref = golden["ov_%s_d%d" % (case, depth_idx)][s]
        assert numpy.array_equal(img > 0, ref > 0)
        if ref.max() > 0:
            big = ref > 1e-6 * ref.max()
            assert (numpy.abs(img - ref)[big] / ref[big]).max() < 1e-5
            assert numpy.abs(img - ref).sum() <= 1e-6 * ref.sum()
    pipe.check_status()


def _rng_for(golden, name):
    fpn = "%s_fpn_normals" % name

    class _Rng:
        def normal(self, *a, **k):
            return golden[fpn]

        def exponential(self, *a, **k):
            raise AssertionError("bleaching times are injected")

    return _Rng() if fpn in golden else numpy.random.RandomState(0)


@pytest.mark.parametrize("name,nframes,tag", FRAME_CASES)
def test_frames_injected_draws(lib, golden, name, nframes, tag):
    import scopyon_gb300 as sg
    tree = case_tree(golden, name)
    cfg = _config_from_tree(tree, cmos_table=golden["cmos_table"].tolist())
    frames = case_frames_draws(golden, name, nframes)
    ids = [int(i) for i in golden["%s_true_ids" % name]]
    bleach = dict(zip(ids, golden["%s_bleach_times" % name])) if len(
        golden["%s_bleach_times" % name]) else {}
    draws = sg.InjectedDraws(bleach=bleach, frames=frames)
    inputs = case_raw_inputs(golden, name)
    sim = sg.EPIFMSimulator(cfg, method="default", rng=_rng_for(golden, name))
    if name == "fa":
        results = [sim.form_image(inputs, full_output=True, draws=draws)]
    else:
        results = list(sim.generate_images(inputs, nframes, full_output=True, draws=draws))
    det = tree["default"]["detector"]["type"]
    for f, (img, info) in enumerate(results):
        e_ref = golden["%s_expectation" % name][f]
        e = info["expectation"]
        big = e_ref > 1e-6 * e_ref.max()
        assert (numpy.abs(e - e_ref)[big] / e_ref[big]).max() < 1e-5
        assert numpy.abs(e - e_ref).sum() <= 1e-6 * e_ref.sum()
        a_ref = golden["%s_adc" % name][f]
        diff = numpy.abs(img.as_array() - a_ref)
        if det == "EMCCD":
            bad = diff > 1e-9
            assert bad.sum() <= max(1, int(1e-4 * diff.size)), bad.sum()
            assert diff.max() <= 1.0
        else:
            assert diff.max() <= 1e-9 * max(1.0, a_ref.max())
        td = numpy.array([info["true_data"][m] for m in ids])
        numpy.testing.assert_allclose(td, golden["%s_true_data" % name][f], rtol=1e-12,
                                      atol=1e-300)
        if "%s_states" % name in golden:
            st = numpy.array([info["fluorescence_states"][m] for m in ids])
            numpy.testing.assert_allclose(st, golden["%s_states" % name][f], rtol=1e-12, atol=0)


def test_emccd_exact_matches_oracle(lib):
    """Exact EMCCD inverse CDF on the device vs the oracle, including E > 709 e-."""
    rng = numpy.random.RandomState(3)
    e = numpy.concatenate([[0.0, 0.01, 0.5, 3.7, 55.0, 333.3, 700.0, 1200.0],
                           rng.uniform(0, 800, 56)])
    u = rng.uniform(size=e.size)
    photons = _dev(e.astype(numpy.float32).astype(numpy.float64))
    out = torch.empty(e.size, dtype=torch.float64, device="cuda")
    status = torch.zeros(4, dtype=torch.int32, device="cuda")
    lib.call("sc_emccd_exact", lib.ptr(photons), 1.0, 0.0, lib.ptr(_dev(u)), e.size, 300.0,
             lib.ptr(out), lib.ptr(status), lib.stream_ptr())
    got = out.cpu().numpy()
    ref = numpy.array([O.emccd_draw(float(numpy.float32(x)), 300, uu) for x, uu in zip(e, u)])
    assert (got != ref).sum() <= 1
    assert numpy.abs(got - ref).max() <= 1
    assert status.cpu().numpy()[0] == 0
