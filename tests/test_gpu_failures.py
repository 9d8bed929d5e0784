"""GPU: failures reported to the host, and invariance to the emitters' order.

Every failure here is made on the host or by a bounded wait that runs out;
none faults, traps or hangs the GPU, and each test checks that the context
still gives correct frames afterwards.

* A non-finite emitter position raises ValueError, as the reference's
  ``math.floor`` does (src/scopyon/_epifm.py:233); a non-finite depth is
  caught on the host before any launch.
* The splat's bounded mbarrier wait: with the test hook that gives each
  warp's first block wait no polls, the wait runs out at once, the copies
  already in flight are drained under the normal bound, status bit 5 is set
  and the host raises SC_ERR_TIMEOUT.
* Permuting the emitters within every sub-step moves the order of the
  footprint sums only: expectations within 1e-5 per pixel (above 1e-6 of the
  maximum), true_data equal per molecule id (rtol 1e-12).
"""

import math

import numpy
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from scopyon_gb300 import _build, _lib
    _build.build()
    return _lib


def _cfg(edge=64, detector="EMCCD"):
    import scopyon_gb300 as sg
    cfg = sg.DefaultConfiguration()
    cfg.update({"default": {"magnification": 100,
                            "detector": {"type": detector, "image_size": [edge, edge],
                                         "exposure_time": 0.01},
                            "light_source": {"angle": 0.0},
                            "effects": {"photo_bleaching": {"switch": False}}}})
    return cfg


def _points(n, edge, seed):
    rng = numpy.random.RandomState(seed)
    half = edge * 160e-9 / 2
    return rng.uniform(-half, half, (n, 2))


def test_nan_position_raises_value_error(lib):
    import scopyon_gb300 as sg
    cfg = _cfg()
    pts = _points(50, 64, 1)
    good, _ = sg.form_image(pts, config=cfg, rng=numpy.random.RandomState(2), full_output=True,
                            device="cuda:0")
    bad = pts.copy()
    bad[17, 0] = numpy.nan
    with pytest.raises(ValueError, match="non-finite"):
        sg.form_image(bad, config=cfg, rng=numpy.random.RandomState(2), device="cuda:0")
    bad = pts.copy()
    bad[3, 1] = numpy.inf
    with pytest.raises(ValueError, match="non-finite"):
        sg.form_image(bad, config=cfg, rng=numpy.random.RandomState(2), device="cuda:0")
    # a NaN depth is caught on the host
    p3 = numpy.column_stack([pts, numpy.zeros(len(pts))])
    p3[5, 2] = numpy.nan
    with pytest.raises(ValueError):
        sg.form_image(p3, config=cfg, rng=numpy.random.RandomState(2), device="cuda:0")
    # the context is still usable and the same inputs give the same frame
    again, _ = sg.form_image(pts, config=cfg, rng=numpy.random.RandomState(2), full_output=True,
                             device="cuda:0")
    numpy.testing.assert_array_equal(again.as_array(), good.as_array())


@pytest.mark.parametrize("bad", ["x", "depth"])
def test_error_surfaces_at_its_frame_in_a_sequence(lib, bad):
    """generate_images reads each frame back while the next one runs.  A
    non-finite x at frame 3 (found by the device) or depth at frame 3 (found
    on the host) still comes out as ValueError at frame 3: frames 0-2 equal
    those of the clean inputs first."""
    import scopyon_gb300 as sg
    cfg = _cfg(edge=48)
    rng = numpy.random.RandomState(5)
    n, sub = 40, 4
    half = 48 * 160e-9 / 2
    pts = numpy.column_stack([rng.uniform(-half, half, (n, 2)), rng.uniform(-1e-7, 1e-7, n),
                              numpy.arange(n), numpy.ones(n)])
    t = numpy.arange(6 * sub + 1) * (0.01 / sub)
    clean = []
    for _ in t:
        pts = pts.copy()
        pts[:, :2] += 2e-8 * rng.standard_normal((n, 2))
        clean.append(pts)
    dirty = [a.copy() for a in clean]
    dirty[3 * sub + 1][7, 0 if bad == "x" else 2] = numpy.nan

    def frames(arrays, k):
        gen = sg.generate_images([(float(a), b) for a, b in zip(t, arrays)], 6, config=cfg,
                                 rng=numpy.random.RandomState(8), device="cuda:0")
        return gen, [next(gen).as_array() for _ in range(k)]

    _, want = frames(clean, 6)
    gen, got = frames(dirty, 3)
    for a, b in zip(got, want):
        numpy.testing.assert_array_equal(a, b)
    with pytest.raises(ValueError):
        next(gen)
    # the context still gives the clean frames
    _, again = frames(clean, 6)
    numpy.testing.assert_array_equal(numpy.array(again), numpy.array(want))


def test_splat_wait_runs_out_and_is_reported(lib):
    """The bulk-copy splat (160 nm pixels, box tables) with no polls for each
    warp's first wait: SC_ERR_TIMEOUT through the status word, then a normal
    frame on the same pipeline equals a fresh pipeline's."""
    from scopyon_gb300.base import _psf_for
    from scopyon_gb300.epifm import EngineConfig, FramePipeline
    cfg = _cfg(edge=128)
    eng = EngineConfig(cfg["default"], rng=numpy.random.RandomState(0))
    pipe = FramePipeline(eng, "cuda:0", psf=_psf_for(eng, torch.device("cuda:0")))
    assert pipe.psf.box_p == 160 and pipe.psf.box_nq == 14  # the bulk-copy kernel's geometry
    n, S = 3000, 4
    parts = numpy.zeros((S, n, 5))
    parts[:, :, 1:3] = _points(n, 128, 3)[None]
    parts[:, :, 3] = numpy.arange(n)
    parts[:, :, 4] = 1.0
    pipe.psf.ensure([0])
    ut = numpy.full(S, 0.01 / S)
    pipe.first_wait_polls = -1
    pipe.run_frame(parts, ut, with_optinfo=False, seed=5)
    torch.cuda.synchronize()
    st = pipe.status.cpu().numpy().copy()
    assert st[0] & 32, st
    with pytest.raises(lib.ScopyonGPUError) as err:
        pipe.check_status()
    assert err.value.code == lib.SC_ERR_TIMEOUT
    assert "ran out" in str(err.value)
    pipe.first_wait_polls = 0
    pipe.run_frame(parts, ut, with_optinfo=False, seed=5)
    img = pipe.expect.cpu().numpy().copy()
    pipe.check_status()
    fresh = FramePipeline(eng, "cuda:0", psf=pipe.psf)
    fresh.run_frame(parts, ut, with_optinfo=False, seed=5)
    numpy.testing.assert_array_equal(fresh.expect.cpu().numpy(), img)
    fresh.check_status()
    assert img.sum() > 0


def test_emitter_permutation_invariance(lib):
    import scopyon_gb300 as sg
    edge, n, S = 256, 4000, 5
    cfg = _cfg(edge=edge, detector="CMOS")
    cfg.update({"default": {"effects": {"photo_bleaching": {"switch": True,
                                                            "half_life": 2 * math.log(2)}},
                            "gpu": {"cmos_noise": "scmos"}}})
    rng = numpy.random.RandomState(9)
    dt = 0.01 / S
    pos = numpy.zeros((S + 1, n, 3))
    pos[0, :, :2] = _points(n, edge, 4)
    pos[0, :, 2] = rng.uniform(-1e-6, 1e-6, n)
    for k in range(S):
        pos[k + 1] = pos[k] + 3e-8 * rng.standard_normal((n, 3))
    ids = numpy.arange(n, dtype=float)
    perm = rng.permutation(n)
    bleach = dict(zip(range(n), rng.exponential(2.0, n)))

    def run(order):
        inputs = [(k * dt, numpy.column_stack([pos[k][order], ids[order], numpy.ones(n)]))
                  for k in range(S + 1)]
        return next(sg.generate_images(inputs, 1, config=cfg, rng=numpy.random.RandomState(1),
                                       full_output=True, device="cuda:0",
                                       draws=sg.InjectedDraws(bleach=bleach)))[1]

    a = run(numpy.arange(n))
    b = run(perm)
    ea, eb = a["expectation"], b["expectation"]
    big = ea > 1e-6 * ea.max()
    assert (numpy.abs(ea - eb)[big] / ea[big]).max() <= 1e-5
    assert not numpy.array_equal(perm, numpy.arange(n))
    for m in range(n):
        numpy.testing.assert_allclose(b["true_data"][m], a["true_data"][m], rtol=1e-12)
        assert b["fluorescence_states"][m] == pytest.approx(a["fluorescence_states"][m],
                                                             rel=1e-12)
