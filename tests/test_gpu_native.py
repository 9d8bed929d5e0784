"""GPU: device trajectories and the native (Philox) random draws.

* exact-mode trajectories equal the reference's sample_inputs bit for bit;
* frames from device trajectories equal the reference's frames (injected
  camera draws), tolerances as in test_gpu_parity;
* Philox Brownian steps: mean-squared displacement per axis within 4 sigma
  of 2 D t; reflecting / periodic boundaries keep particles in the box;
* native camera models: per-pixel mean and variance of the photo-electron
  signal within 4 standard errors of the model's moments, and a
  Kolmogorov-Smirnov test of the sCMOS / CCD read noise.
"""

import json

import numpy
import pytest

torch = pytest.importorskip("torch")
from golden_cases import case_frames_draws, case_tree  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sg():
    from scopyon_gb300 import _build
    _build.build()
    import scopyon_gb300
    return scopyon_gb300


def test_exact_trajectories_match_reference(sg, golden):
    t = numpy.arange(7) * 0.5e-3
    traj = sg.sample_inputs(t, N=5, lower=[-1e-6, -2e-6, -0.5e-6], upper=[1e-6, 2e-6, 0.5e-6],
                            D=0.1e-12, ndim=3, rng=numpy.random.RandomState(5), exact=True)
    pts = numpy.array([p for _, p in traj])
    numpy.testing.assert_array_equal(pts, golden["samp3_pts"])
    traj = sg.sample_inputs(t[:4], N=4, lower=-3e-6, upper=3e-6, D=[0.2e-12, 0.05e-12], ndim=2,
                            rng=numpy.random.RandomState(9), exact=True)
    numpy.testing.assert_array_equal(numpy.array([p for _, p in traj]), golden["samp2_pts"])


@pytest.mark.parametrize("name,nframes,seed,n,lower,upper,D", [
    ("fb", 3, 3, 9, [-1.5e-6, -1.5e-6, -0.4e-6], [1.5e-6, 1.5e-6, 0.4e-6], 0.2e-12),
    ("fd", 2, 8, 5, [-1.0e-6, -1.0e-6, 0.0], [1.0e-6, 1.0e-6, 0.2e-6], 0.5e-12),
])
def test_device_frames_match_reference(sg, golden, name, nframes, seed, n, lower, upper, D):
    tree = json.loads(json.dumps(case_tree(golden, name)))
    tree["default"]["gpu"] = {"cmos_table": golden["cmos_table"].tolist()}
    cfg = sg.Configuration(yaml=tree)
    times = golden["%s_input_t" % name]
    traj = sg.sample_inputs(times, N=n, lower=lower, upper=upper, D=D, ndim=3,
                            rng=numpy.random.RandomState(seed), exact=True)
    ids = [int(i) for i in golden["%s_true_ids" % name]]
    bleach = dict(zip(ids, golden["%s_bleach_times" % name]))
    draws = sg.InjectedDraws(bleach=bleach, frames=case_frames_draws(golden, name, nframes))
    sim = sg.EPIFMSimulator(cfg, method="default", rng=numpy.random.RandomState(0))
    results = list(sim.generate_images(traj, nframes, full_output=True, draws=draws))
    for f, (img, info) in enumerate(results):
        e_ref = golden["%s_expectation" % name][f]
        big = e_ref > 1e-6 * e_ref.max()
        assert (numpy.abs(info["expectation"] - e_ref)[big] / e_ref[big]).max() < 1e-5
        a_ref = golden["%s_adc" % name][f]
        diff = numpy.abs(img.as_array() - a_ref)
        if tree["default"]["detector"]["type"] == "EMCCD":
            assert (diff > 1e-9).sum() <= 1 and diff.max() <= 1.0
        else:
            assert diff.max() <= 1e-9 * a_ref.max()
        td = numpy.array([info["true_data"][m] for m in ids])
        numpy.testing.assert_allclose(td, golden["%s_true_data" % name][f], rtol=1e-12)
        st = numpy.array([info["fluorescence_states"][m] for m in ids])
        numpy.testing.assert_allclose(st, golden["%s_states" % name][f], rtol=1e-12, atol=0)


def test_philox_diffusion_msd(sg):
    n, steps, dt, D = 20000, 50, 1e-3, 0.3e-12
    traj = sg.sample_inputs(numpy.arange(steps + 1) * dt, N=n, lower=0.0, upper=0.0, D=D, ndim=3,
                            rng=numpy.random.RandomState(1))
    end = traj.copy().materialize(steps)
    disp = end[:, :3]
    var = 2 * D * steps * dt
    for d in range(3):
        msd = (disp[:, d] ** 2).mean()
        # chi-square with n dof: mean var, sd var * sqrt(2/n)
        assert abs(msd / var - 1) < 4 * numpy.sqrt(2.0 / n), (d, msd / var)
        assert abs(disp[:, d].mean()) < 4 * numpy.sqrt(var / n)
    # consecutive steps are independent
    a = traj.copy().materialize(1)[:, 0]
    b = traj.copy().materialize(2)[:, 0] - a
    assert abs(numpy.corrcoef(a, b)[0, 1]) < 4 / numpy.sqrt(n)


@pytest.mark.parametrize("boundary", ["reflecting", "periodic"])
def test_boundaries_confine(sg, boundary):
    lo, hi = -0.5e-6, 0.5e-6
    traj = sg.sample_inputs(numpy.arange(201) * 1e-3, N=4000, lower=lo, upper=hi, D=1e-12, ndim=3,
                            rng=numpy.random.RandomState(2), boundary=boundary)
    end = traj.copy().materialize(200)[:, :3]
    assert end.min() >= lo and end.max() <= hi
    # after many box-crossing times the density is uniform
    hist, _ = numpy.histogram(end[:, 0], bins=10, range=(lo, hi))
    expected = len(end) / 10
    chi2 = ((hist - expected) ** 2 / expected).sum()
    assert chi2 < 30  # 9 dof, p ~ 4e-4


def _camera_stats(sg, det, gpu, photons, n_frames=40, seed=3):
    cfg = sg.DefaultConfiguration()
    cfg.update({"default": {
        "magnification": 100,
        "detector": {"type": det, "image_size": [64, 64], "exposure_time": 0.01},
        "effects": {"background": {"switch": True, "mean": photons},
                    "photo_bleaching": {"switch": False}},
        # fullwell = 2^16 - offset makes the ADC gain exactly 1 e- per count
        "analog_to_digital_converter": {"bit": 16, "offset": 2000, "fullwell": 63536},
        "gpu": gpu}})
    sim = sg.EPIFMSimulator(cfg, method="default", rng=numpy.random.RandomState(seed))
    far = numpy.array([[1.0, 1.0]])  # one emitter far outside the field: background only
    imgs = [img.as_array() for img in sim.generate_images(far, n_frames)]
    eng = sim.base()
    return numpy.array(imgs), eng


def test_native_ccd_moments_and_noise(sg):
    imgs, eng = _camera_stats(sg, "CCD", {}, photons=50.0)
    e = eng.qe * 50.0
    electrons = (imgs - eng.offset) * eng.gain
    m, v = electrons.mean(), electrons.var()
    n = electrons.size
    var_model = e + eng.readout_noise ** 2
    assert abs(m - e) < 4 * numpy.sqrt(var_model / n)
    assert abs(v / var_model - 1) < 4 * numpy.sqrt(2.0 / n) * 1.5


def test_native_emccd_moments(sg):
    imgs, eng = _camera_stats(sg, "EMCCD", {}, photons=20.0)
    e, g = eng.qe * 20.0, eng.emgain
    electrons = (imgs - eng.offset) * eng.gain
    m, v = electrons.mean(), electrons.var()
    n = electrons.size
    var_model = 2 * g * g * e + eng.readout_noise ** 2
    assert abs(m / (g * e) - 1) < 4 * numpy.sqrt(var_model / n) / (g * e) + 1e-3
    assert abs(v / var_model - 1) < 0.05


def test_native_scmos_per_pixel_sigma(sg):
    imgs, eng = _camera_stats(sg, "CMOS", {"cmos_noise": "scmos", "scmos_readout_median": 1.5,
                                           "scmos_readout_sigma": 0.4}, photons=30.0, n_frames=80)
    e = eng.qe * 30.0
    electrons = (imgs - eng.offset) * eng.gain
    m = electrons.mean()
    assert abs(m - e) < 4 * numpy.sqrt((e + 4) / electrons.size)
    # per-pixel variance ~ e + sigma_ij^2 with lognormal(ln 1.5, 0.4) sigmas: median excess ~2.25
    pv = electrons.var(axis=0, ddof=1) - e
    assert 1.5 < numpy.median(pv) < 3.2


@pytest.mark.parametrize("kind", ["EMCCD", "CCD", "CMOS_TABLE", "SCMOS"])
def test_camera_draws_do_not_depend_on_the_grouping(sg, kind):
    """A pixel's native draws come from its own Philox stream: frames of
    different sizes (so the grid-stride loop hands each pixel to a different
    thread and iteration) give the same counts, bit for bit, on the pixels
    they share.  Photons mix empty pixels, table means (below 256) and bright
    pixels on the PTRS fallback."""
    from scopyon_gb300 import _lib
    from scopyon_gb300._lib import call, ptr, stream_ptr
    dev = torch.device("cuda")
    nh = 1024
    n_big = 2048 * nh
    g = torch.Generator(dev).manual_seed(11)
    u = torch.rand(n_big, device=dev, generator=g)
    photons = torch.where(u < 0.3, torch.zeros_like(u),
                          torch.where(u < 0.7, 15.0 * torch.rand(n_big, device=dev, generator=g),
                                      15.0 + 500.0 * torch.rand(n_big, device=dev, generator=g)))
    offset_f = torch.round(100.0 + 5.0 * torch.randn(n_big, device=dev, generator=g))
    inv_gain_f = (4096.0 - offset_f) / 30000.0
    sigma = torch.exp(0.4 + 0.4 * torch.randn(n_big, device=dev, generator=g))
    tv = torch.linspace(0.5, 5.0, 16, dtype=torch.float64, device=dev)
    tc = torch.cumsum(torch.full((16,), 1.0 / 16, dtype=torch.float64, device=dev), 0)
    tc[-1] = 1.0
    status = torch.zeros(_lib.STATUS_WORDS, dtype=torch.int32, device=dev)
    cam = {"EMCCD": _lib.CAM_EMCCD, "CCD": _lib.CAM_CCD, "CMOS_TABLE": _lib.CAM_CMOS_TABLE,
           "SCMOS": _lib.CAM_SCMOS}[kind]

    def run(nw):
        n = nw * nh
        cp = _lib.CameraParams()
        cp.nw, cp.nh, cp.camera, cp.exact, cp.rounding, cp.bit = nw, nh, cam, 0, 1, 16
        cp.qe, cp.background, cp.readout_noise = 0.9, 2.0, 3.0
        cp.emgain, cp.fullwell, cp.offset0, cp.gain0 = 300.0, 6.0e5, 100.0, 10.0
        cp.table_n = 16 if kind == "CMOS_TABLE" else 0
        cp.seed, cp.counter = 1234567, 5
        cp.d_poisson_table = _lib.poisson_table(dev).data_ptr()
        expect = torch.empty(n, dtype=torch.float32, device=dev)
        adc = torch.empty(n, dtype=torch.float64, device=dev)
        call("sc_camera", cp, ptr(photons), None, None, ptr(offset_f), ptr(inv_gain_f),
             ptr(sigma) if kind == "SCMOS" else None, ptr(tv), ptr(tc), None, None, None,
             ptr(expect), ptr(adc), None, ptr(status), stream_ptr())
        torch.cuda.synchronize()
        return expect.cpu().numpy(), adc.cpu().numpy()

    e_small, a_small = run(300)   # 307,200 px: about one pixel per thread
    e_mid, a_mid = run(1024)      # 1,048,576 px: several pixels per thread
    e_big, a_big = run(2048)      # 2,097,152 px
    assert int(status[0].item()) == 0
    k = len(a_small)
    numpy.testing.assert_array_equal(e_mid[:k], e_small)
    numpy.testing.assert_array_equal(a_mid[:k], a_small)
    numpy.testing.assert_array_equal(e_big[:len(e_mid)], e_mid)
    numpy.testing.assert_array_equal(a_big[:len(a_mid)], a_mid)
    assert len(numpy.unique(a_big)) > 100


def test_poisson_sampler_distribution(sg):
    """Photo-electron counts of the CCD path (read noise off) follow Poisson(E): chi-square."""
    from scipy import stats
    cfg = sg.DefaultConfiguration()
    for photons in (3.0, 40.0, 400.0):
        cfg.update({"default": {
            "magnification": 100,
            "detector": {"type": "CCD", "image_size": [64, 64], "readout_noise": 0},
            "effects": {"background": {"switch": True, "mean": photons},
                        "photo_bleaching": {"switch": False}},
            "analog_to_digital_converter": {"bit": 16, "offset": 2000, "fullwell": 63536}}})
        sim = sg.EPIFMSimulator(cfg, method="default", rng=numpy.random.RandomState(4))
        imgs = numpy.array([i.as_array() for i in sim.generate_images(numpy.array([[1.0, 1.0]]), 10)])
        eng = sim.base()
        counts = numpy.rint((imgs - eng.offset) * eng.gain).astype(int).ravel()
        lam = eng.qe * photons
        lo, hi = int(max(0, lam - 4 * numpy.sqrt(lam))), int(lam + 4 * numpy.sqrt(lam)) + 1
        edges = numpy.arange(lo, hi + 1)
        obs = numpy.array([(counts == k).sum() for k in edges[:-1]])
        exp = stats.poisson.pmf(edges[:-1], lam) * counts.size
        keep = exp > 20
        chi2 = (((obs - exp) ** 2) / exp)[keep].sum()
        dof = keep.sum() - 1
        assert stats.chi2.sf(chi2, dof) > 1e-4, (photons, chi2, dof)


def test_frame_graph_replay_matches_eager(sg):
    """Frames replayed from one captured CUDA graph equal eagerly launched
    frames, also with 2, 3, 8 and 16 frames per replay and with the records
    running up to 2 or 3 frames ahead, every frame's outputs kept."""
    from scopyon_gb300.base import _psf_for
    from scopyon_gb300.epifm import EngineConfig, FrameGraph, FramePipeline
    cfg = sg.DefaultConfiguration()
    cfg.update({"default": {
        "magnification": 100, "light_source": {"angle": 0.0},
        "detector": {"type": "CMOS", "image_size": [48, 40], "exposure_time": 0.004},
        "effects": {"photo_bleaching": {"switch": True, "half_life": 0.01}},
        "gpu": {"cmos_noise": "scmos"}}})
    outs = []
    # (graph, frames per replay, record and bin buffer sets)
    cases = ((False, 1, 2), (True, 1, 2), (False, 2, 2), (True, 2, 2), (True, 3, 2),
             (True, 8, 2), (True, 16, 2), (True, 3, 3), (True, 16, 3))
    n_frames = 48
    for use_graph, per_step, sets in cases:
        rng = numpy.random.RandomState(6)
        eng = EngineConfig(cfg["default"], rng=rng)
        pipe = FramePipeline(eng, "cuda", psf=_psf_for(eng, torch.device("cuda")))
        pipe.scmos_sigma_map(rng)
        t = numpy.arange(n_frames * 4 + 1) * 1e-3
        traj = sg.sample_inputs(t, N=300, lower=[-3e-6, -3e-6, -0.3e-6], upper=[3e-6, 3e-6, 0.3e-6],
                                D=0.5e-12, ndim=3, rng=rng, boundary="reflecting")
        pipe.psf.ensure(list(range(0, 700)))
        pipe.ensure_slots(300)
        pipe.budget[:300].copy_(torch.from_numpy(rng.exponential(0.02, 300) * eng.n_emit0))
        fg = FrameGraph(pipe, traj, 4, 1e-3, seed=77, use_graph=use_graph,
                        frames_per_step=per_step)
        fg.record_sets = sets
        frames = []
        for _ in range(n_frames // per_step):
            fg.step()
            # every frame of a step keeps its own outputs, the last in pipe.adc32
            assert fg.outputs[-1][1] is pipe.adc32
            frames.extend(adc.cpu().numpy().copy() for _, adc in fg.outputs)
        pipe.check_status()
        pos = traj._pos.cpu().numpy().copy()
        outs.append((numpy.array(frames), pos))
    numpy.testing.assert_array_equal(outs[0][0], outs[1][0])
    assert outs[0][0].std(axis=0).max() > 0  # frames differ from one another
    # several frames per step (each frame's records overlapping the previous
    # frame's splat) give the same frames and trajectories
    for k in range(2, len(cases)):
        numpy.testing.assert_array_equal(outs[k][0], outs[0][0], err_msg=str(cases[k]))
        numpy.testing.assert_array_equal(outs[k][1], outs[0][1])


@pytest.mark.parametrize("angle,bleach,ndim", [(None, False, 3), (None, True, 3), (0.0, True, 3),
                                               (None, True, 2)])
def test_fused_native_physics_matches_separate_pass(sg, angle, bleach, ndim):
    """sc_native_records (diffusion, physics and footprints in one pass) equals
    sc_diffuse_steps followed by sc_emitter_steps on the same Philox trajectory:
    identical expectation images.  TIRF with depth (the default angle), with and
    without photobleaching (a half-life short enough that emitters bleach inside
    the frames), EPI (angle 0) and a flat field (ndim 2: the excitation is the
    same for every emitter)."""
    from scopyon_gb300.base import _psf_for
    from scopyon_gb300.epifm import EngineConfig, FrameGraph, FramePipeline
    cfg = sg.DefaultConfiguration()
    upd = {"magnification": 100,
           "detector": {"type": "EMCCD", "image_size": [40, 40], "exposure_time": 0.004},
           "effects": {"photo_bleaching": {"switch": bleach, "half_life": 0.006}}}
    if angle is not None:
        upd["light_source"] = {"angle": angle}
    cfg.update({"default": upd})
    t = numpy.arange(4 * 4 + 1) * 1e-3
    lo, hi = [-2.5e-6, -2.5e-6, -0.2e-6][:ndim], [2.5e-6, 2.5e-6, 0.2e-6][:ndim]
    traj = sg.sample_inputs(t, N=200, lower=lo, upper=hi, D=0.4e-12, ndim=ndim,
                            rng=numpy.random.RandomState(12))
    eng = EngineConfig(cfg["default"])
    pipe = FramePipeline(eng, "cuda", psf=_psf_for(eng, torch.device("cuda")))
    pipe.psf.ensure(list(range(0, 800)))
    if bleach:  # the budgets the separate pass draws first from its generator
        beta = eng.half_life / numpy.log(2.0)
        times_b = numpy.random.RandomState(0).exponential(scale=beta, size=200)
        pipe.ensure_slots(200)
        pipe.budget[:200].copy_(torch.from_numpy(times_b * eng.n_emit0))
    fg = FrameGraph(pipe, traj.copy(), 4, 1e-3, seed=3, use_graph=False)
    fused = []
    for _ in range(4):
        fg.step()
        fused.append(pipe.expect.cpu().numpy().copy())
    budget = pipe.budget[:200].cpu().numpy().copy()
    sim = sg.EPIFMSimulator(cfg, method="default", rng=numpy.random.RandomState(0))
    sep = [info for _, info in sim.generate_images(traj.copy(), 4, full_output=True)]
    for a, info in zip(fused, sep):
        numpy.testing.assert_array_equal(a.reshape(40, 40).astype(float), info["expectation"])
    if bleach:
        # the same emitters bleached; the budgets left agree to rounding (the
        # frame graph's sub-step length is 1 ms, the generator's the difference
        # of two sample times)
        states = sep[-1]["fluorescence_states"]
        sep_budget = numpy.array([states[m] for m in sorted(states)])
        numpy.testing.assert_array_equal(budget == 0, sep_budget == 0)
        numpy.testing.assert_allclose(budget, sep_budget, rtol=1e-12, atol=0)
        assert (budget == 0).any() and (budget > 0).any()  # some emitters bleached, not all


@pytest.mark.parametrize("pin_limit", [None, 0])
def test_host_inputs_fast_path_matches_general_path(sg, pin_limit, monkeypatch):
    """Host trajectories with the same ids at every sub-step take a fast path
    (full_output=False): uploads from one pinned block of all the formatted
    inputs, or (with no room for the block) per-frame staging on host
    threads, each frame read back while the next one runs.  The frames equal
    those of the general path (full_output=True), with bleaching on."""
    from scopyon_gb300 import base
    if pin_limit is not None:
        monkeypatch.setattr(base, "_PIN_LIMIT", pin_limit)
    cfg = sg.DefaultConfiguration()
    cfg.update({"default": {
        "magnification": 100,
        "detector": {"type": "EMCCD", "image_size": [48, 40], "exposure_time": 0.004},
        "effects": {"photo_bleaching": {"switch": True, "half_life": 0.01}}}})
    t = numpy.arange(5 * 4 + 1) * 1e-3
    inputs = [(float(a), p) for a, p in sg.sampling.sample_inputs(
        t, N=150, lower=[-3e-6, -3e-6, -0.2e-6], upper=[3e-6, 3e-6, 0.2e-6], D=0.3e-12, ndim=3,
        rng=numpy.random.RandomState(2), exact=True)]
    outs = []
    for full in (True, False):
        gen = sg.generate_images(inputs, 5, config=cfg, rng=numpy.random.RandomState(9),
                                 full_output=full)
        frames = [(img if not full else img[0]).as_array() for img in gen]
        outs.append(numpy.array(frames))
    numpy.testing.assert_array_equal(outs[0], outs[1])
    assert outs[0].std(axis=0).max() > 0


def test_host_rows_graph_recaptures_when_the_psf_tables_grow(sg, monkeypatch):
    """Native frames from a pinned block of host rows replay captured graphs
    (records, binning, splat, camera), with each frame's rows uploaded on a
    copy stream while the frame before runs.  When the depths reach new PSF
    keys mid-sequence, the tables are reallocated and the graphs captured
    again; every frame still equals the general path's (no graphs) bit for
    bit."""
    from scopyon_gb300 import base
    monkeypatch.setattr(base, "_PSF_CACHE", {})  # tables that start empty and grow
    made = []

    class Recording(base.HostRowsGraph):
        def __init__(self, *a, **k):
            super().__init__(*a, **k)
            made.append(self)

    monkeypatch.setattr(base, "HostRowsGraph", Recording)
    cfg = sg.DefaultConfiguration()
    cfg.update({"default": {
        "magnification": 100,
        "detector": {"type": "EMCCD", "image_size": [56, 48], "exposure_time": 0.004}}})
    rng = numpy.random.RandomState(4)
    n, n_frames = 200, 6
    ids = numpy.arange(n, dtype=float)
    inputs = []
    for k in range(n_frames * 4 + 1):
        z_half = 0.05e-6 if k < 8 else 0.6e-6  # frames 2 on reach deeper keys
        xyz = numpy.column_stack([rng.uniform(-3e-6, 3e-6, n), rng.uniform(-3e-6, 3e-6, n),
                                  rng.uniform(-z_half, z_half, n)])
        inputs.append((k * 1e-3, numpy.hstack([xyz, ids[:, None], numpy.ones((n, 1))])))
    outs = []
    for full in (False, True):
        gen = sg.generate_images(inputs, n_frames, config=cfg, rng=numpy.random.RandomState(5),
                                 full_output=full)
        outs.append(numpy.array([(img[0] if full else img).as_array() for img in gen]))
    assert len(made) == 1 and made[0].captures >= 2
    numpy.testing.assert_array_equal(outs[0], outs[1])
    assert outs[0].std(axis=0).max() > 0


@pytest.mark.parametrize("boundary,ndim", [("reflecting", 3), ("periodic", 3), ("none", 2)])
def test_native_rows_layouts_agree(sg, boundary, ndim):
    """Native (Philox) trajectories move in FP32: every position is an FP32
    value.  The 16-byte FP32 rows (layout 1) hold the same values as the FP64
    [depth, x, y, id, state] rows (layout 0), and a launch without rows
    leaves the particles where a launch with rows does."""
    n, n_sub = 1000, 7
    t = numpy.arange(3 * n_sub + 1) * 1e-3
    lo, hi = [-2e-6, -2e-6, -0.3e-6][:ndim], [2e-6, 2e-6, 0.3e-6][:ndim]
    traj = sg.sample_inputs(t, N=n, lower=lo, upper=hi, D=0.5e-12, ndim=ndim,
                            rng=numpy.random.RandomState(8), boundary=boundary)
    a, b, c = traj.copy(), traj.copy(), traj.copy()
    rows0 = torch.empty(n_sub * n * 5, dtype=torch.float64, device="cuda")
    rows1 = torch.empty(n_sub * n * 4, dtype=torch.float32, device="cuda")
    for g0 in (0, n_sub, 2 * n_sub):
        a.run(g0, n_sub, rows0, layout=0)
        b.run(g0, n_sub, rows1, layout=1)
        c.run(g0, n_sub, None)
        r0 = rows0.view(n_sub, n, 5).cpu().numpy()
        r1 = rows1.view(n_sub, n, 4).cpu().numpy().astype(numpy.float64)
        numpy.testing.assert_array_equal(r0[:, :, :3], r1[:, :, :3])
        assert (r1[:, :, 3] == 0).all()
        numpy.testing.assert_array_equal(r0[:, :, 3], numpy.broadcast_to(numpy.arange(n), (n_sub, n)))
        numpy.testing.assert_array_equal(r0[:, :, 4], 1.0)
        pa, pb, pc = (x._pos.cpu().numpy() for x in (a, b, c))
        numpy.testing.assert_array_equal(pa, pb)
        numpy.testing.assert_array_equal(pa, pc)
        numpy.testing.assert_array_equal(pa, pa.astype(numpy.float32).astype(numpy.float64))
        assert (r0[1:, :, 1] != r0[:-1, :, 1]).mean() > 0.9  # the particles move
    if boundary == "reflecting":
        for d in range(ndim):
            assert (pa[:, d] >= numpy.float32(lo[d])).all() and (pa[:, d] <= numpy.float32(hi[d])).all()


def test_device_frames_from_fp32_rows_equal_fp64_rows(sg, monkeypatch):
    """generate_images on native device trajectories reads the 16-byte FP32
    rows; forcing the FP64 rows gives the same frames, bit for bit."""
    from scopyon_gb300.sampling import DeviceTrajectories
    cfg = sg.DefaultConfiguration()
    cfg.update({"default": {"magnification": 100,
                            "detector": {"type": "EMCCD", "image_size": [48, 48],
                                         "exposure_time": 0.004},
                            "effects": {"photo_bleaching": {"switch": True, "half_life": 0.01}}}})
    t = numpy.arange(5 * 4 + 1) * 1e-3
    traj = sg.sample_inputs(t, N=300, lower=[-3e-6, -3e-6, -0.2e-6], upper=[3e-6, 3e-6, 0.2e-6],
                            D=0.3e-12, ndim=3, rng=numpy.random.RandomState(21))
    assert traj.compact_rows({"scale": 1.0})

    def frames():
        sim = sg.EPIFMSimulator(cfg, method="default", rng=numpy.random.RandomState(2))
        return [(img.as_array(), info["expectation"], info["fluorescence_states"])
                for img, info in sim.generate_images(traj.copy(), 4, full_output=True)]

    fp32 = frames()
    monkeypatch.setattr(DeviceTrajectories, "compact_rows", lambda self, transform=None: False)
    fp64 = frames()
    for (a1, e1, s1), (a0, e0, s0) in zip(fp32, fp64):
        numpy.testing.assert_array_equal(e1, e0)
        numpy.testing.assert_array_equal(a1, a0)
        assert s1 == s0
    assert fp32[0][1].max() > 0


def _philox4x32_10(ctr, key):
    """Philox4x32-10 of one counter (four uint32) and key (two uint32), as the
    kernels draw it (Salmon et al., SC'11)."""
    x, y, z, w = (int(v) & 0xffffffff for v in ctr)
    k0, k1 = (int(v) & 0xffffffff for v in key)
    for _ in range(10):
        p0, p1 = 0xD2511F53 * x, 0xCD9E8D57 * z
        x, y, z, w = ((p1 >> 32) ^ y ^ k0, p1 & 0xffffffff, (p0 >> 32) ^ w ^ k1,
                      p0 & 0xffffffff)
        k0, k1 = (k0 + 0x9E3779B9) & 0xffffffff, (k1 + 0xBB67AE85) & 0xffffffff
    return x, y, z, w


def test_box_muller_radius_at_the_largest_uniform(sg):
    """A Philox word whose top 24 bits are all set gives the uniform 1.0 (the
    24-bit uniform plus half a step rounds up), so the Box-Muller radius
    sqrt(-2 ln u) is 0.  The seeds below were found by searching the key space
    for such a word: the camera's read-noise word of pixel 0 (counter 1) and
    the first radius of particle 0's normals at step 0.  The draws stay
    finite and the normals 0."""
    from scopyon_gb300 import _lib
    from scopyon_gb300._lib import call, ptr, stream_ptr
    from scopyon_gb300.sampling import DeviceTrajectories
    cam_seed, dif_seed = 2656475, 14960767
    assert _philox4x32_10((0, 1, 0, 0), (cam_seed, 0))[2] >> 8 == 0xFFFFFF
    assert _philox4x32_10((0, 0, 0, 0x5d1ff05e), (dif_seed, 0))[0] >> 8 == 0xFFFFFF
    dev = torch.device("cuda")
    ph = torch.zeros(2, dtype=torch.float32, device=dev)
    adc = torch.empty(2, dtype=torch.float64, device=dev)
    status = torch.zeros(_lib.STATUS_WORDS, dtype=torch.int32, device=dev)
    cp = _lib.CameraParams()
    cp.nw, cp.nh, cp.camera, cp.exact, cp.rounding, cp.bit = 1, 2, _lib.CAM_CCD, 0, 0, 16
    cp.qe, cp.background, cp.readout_noise, cp.emgain = 1.0, 0.0, 50.0, 1.0
    cp.fullwell, cp.offset0, cp.gain0 = 60000.0, 100.0, 1.0
    cp.seed, cp.counter = cam_seed, 1
    cp.d_poisson_table = _lib.poisson_table(dev).data_ptr()
    call("sc_camera", cp, ptr(ph), None, None, None, None, None, None, None, None, None, None,
         None, ptr(adc), None, ptr(status), stream_ptr())
    a = adc.cpu().numpy()
    assert int(status[0]) == 0
    assert numpy.isfinite(a).all()
    assert abs(a[0] - 100.0) < 1e-6  # no photons, no read noise: the offset
    pts = numpy.array([[0.0, 0.0, 0.0, 0.0, 1.0], [1e-7, 1e-7, 0.0, 1.0, 1.0]])
    traj = DeviceTrajectories([0.0, 1e-3, 2e-3], pts, 1e-12, 3, dif_seed, device="cuda")
    end = traj.copy().materialize(1)
    assert numpy.isfinite(end).all()
    assert abs(end[0, 0]) < 1e-18 and abs(end[0, 1]) < 1e-18  # radius 0: no move in x, y
    assert end[0, 2] != 0.0 and end[1, 0] != float(numpy.float32(1e-7))  # the others move


def test_register_box_kernel_equals_bulk_copy_ring(sg):
    """The box splat's register form (16-byte loads, stages 0) adds the same
    values in the same order as the bulk-copy ring: for the same tiles and
    warps, equal expectations bit for bit (8x8 and 16x16 tiles), including
    footprints clipped by the image's low edges (emitters past the field);
    other tilings group the sums differently and agree to FP32 rounding."""
    from scopyon_gb300.base import _psf_for
    from scopyon_gb300.epifm import EngineConfig, FrameGraph, FramePipeline
    cfg = sg.DefaultConfiguration()
    cfg.update({"default": {"magnification": 100,
                            "detector": {"type": "EMCCD", "image_size": [200, 136],
                                         "exposure_time": 0.004},
                            "light_source": {"angle": 0.0}}})
    t = numpy.arange(4 * 4 + 1) * 1e-3
    # reflecting walls keep the depths within the keys built below
    traj = sg.sample_inputs(t, N=3000, lower=[-17e-6, -12e-6, -0.3e-6],
                            upper=[17e-6, 12e-6, 0.3e-6], D=0.4e-12, ndim=3,
                            rng=numpy.random.RandomState(12), boundary="reflecting")
    eng = EngineConfig(cfg["default"])
    out = {}
    for tile, warps, stages in ((8, 4, 4), (8, 4, 0), (16, 8, 4), (16, 8, 0)):
        pipe = FramePipeline(eng, "cuda", psf=_psf_for(eng, torch.device("cuda")))
        pipe.psf.ensure(list(range(0, 400)))
        pipe.set_tiles(tile, warps, stages)
        fg = FrameGraph(pipe, traj.copy(), 4, 1e-3, seed=3, use_graph=False)
        frames = []
        for _ in range(4):
            fg.step()
            frames.append(pipe.expect.cpu().numpy().copy())
        pipe.check_status()
        out[(tile, warps, stages)] = numpy.array(frames)
    ref = out[(8, 4, 4)]
    assert ref.max() > 0
    numpy.testing.assert_array_equal(out[(8, 4, 0)], ref)
    numpy.testing.assert_array_equal(out[(16, 8, 0)], out[(16, 8, 4)])
    assert numpy.abs(out[(16, 8, 0)] - ref).max() <= 1e-6 * ref.max()


def test_frame_graph_checkpoint_resumes_the_same_frames(sg, tmp_path):
    """A frame graph's checkpoint (positions and classes of the trajectories,
    photon budgets, frame counter) pickled to disk and loaded into a new
    pipeline, or back into the same captured graph, continues with the
    frames that followed it, bit for bit, bleaching included."""
    import pickle
    from scopyon_gb300.base import _psf_for
    from scopyon_gb300.epifm import EngineConfig, FrameGraph, FramePipeline
    cfg = sg.DefaultConfiguration()
    cfg.update({"default": {"magnification": 100,
                            "detector": {"type": "EMCCD", "image_size": [96, 80],
                                         "exposure_time": 0.004},
                            "effects": {"photo_bleaching": {"switch": True, "half_life": 0.01}}}})
    t = numpy.arange(9 * 4 + 1) * 1e-3
    traj = sg.sample_inputs(t, N=1500, lower=[-6e-6, -5e-6, -0.2e-6], upper=[6e-6, 5e-6, 0.2e-6],
                            D=0.4e-12, ndim=3, rng=numpy.random.RandomState(21),
                            boundary="reflecting")
    eng = EngineConfig(cfg["default"])
    budget0 = numpy.random.RandomState(22).exponential(0.01 / numpy.log(2.0), 1500) * eng.n_emit0

    def make(k):
        pipe = FramePipeline(eng, "cuda", psf=_psf_for(eng, torch.device("cuda")))
        pipe.psf.ensure(list(range(0, 300)))
        pipe.ensure_slots(1500)
        pipe.budget[:1500].copy_(torch.from_numpy(budget0))
        return FrameGraph(pipe, traj.copy(), 4, 1e-3, seed=11, frames_per_step=k)

    def run(fg, n):
        out = []
        for _ in range(n):
            fg.step()
            out.append(fg.pipe.adc32.cpu().numpy().copy())
        fg.pipe.check_status()
        return numpy.array(out)

    for k in (1, 2):
        fg = make(k)
        run(fg, 2)
        path = tmp_path / ("state%d.pkl" % k)
        path.write_bytes(pickle.dumps(fg.state_dict()))
        after = run(fg, 3)
        state = pickle.loads(path.read_bytes())
        fg2 = make(k)
        fg2.load_state_dict(state)
        numpy.testing.assert_array_equal(run(fg2, 3), after)
        fg.load_state_dict(state)  # back into the graph that ran on
        numpy.testing.assert_array_equal(run(fg, 3), after)
        assert after.std() > 0
        b = fg.pipe.budget[:1500].cpu().numpy()
        assert (b == 0).any() and (b > 0).any()  # some emitters bleached, not all
    with pytest.raises(ValueError, match="another seed"):
        FrameGraph(make(1).pipe, traj.copy(), 4, 1e-3, seed=12).load_state_dict(state)


def test_nvtx_ranges_leave_the_frames_unchanged(sg, monkeypatch):
    """With NVTX ranges on (scopyon/records, bins, splat, camera around the
    launches) the frames are those with them off, bit for bit."""
    cfg = sg.DefaultConfiguration()
    cfg.update({"default": {"magnification": 100,
                            "detector": {"type": "EMCCD", "image_size": [48, 40],
                                         "exposure_time": 0.004}}})
    t = numpy.arange(3 * 4 + 1) * 1e-3
    inputs = [(float(a), p) for a, p in sg.sampling.sample_inputs(
        t, N=150, lower=[-3e-6, -3e-6, -0.2e-6], upper=[3e-6, 3e-6, 0.2e-6], D=0.3e-12, ndim=3,
        rng=numpy.random.RandomState(2), exact=True)]
    outs = []
    for on in ("0", "1"):
        monkeypatch.setenv("SCOPYON_GB300_NVTX", on)
        gen = sg.generate_images(inputs, 3, config=cfg, rng=numpy.random.RandomState(9))
        outs.append(numpy.array([img.as_array() for img in gen]))
    numpy.testing.assert_array_equal(outs[0], outs[1])


def test_l2_fetch_hint_values(sg):
    """The L2 fetch granularity hint takes 0, 32, 64 and 128 bytes."""
    from scopyon_gb300 import _lib
    for b in (0, 32, 64, 128, 32):
        _lib.call("sc_set_l2_fetch_granularity", b)
    with pytest.raises(ValueError, match="48 bytes"):  # SC_ERR_ARG
        _lib.call("sc_set_l2_fetch_granularity", 48)


@pytest.mark.parametrize("det,cmos_noise", [("EMCCD", None), ("CCD", None), ("CMOS", "scmos")])
def test_merge_camera_equals_merge_then_camera(sg, det, cmos_noise):
    """sc_merge_camera (the splat's merge inside the camera pass) gives the
    expectation and ADC counts of sc_splat with its merge followed by
    sc_camera, bit for bit, over frames of a frame graph (and the trajectories
    and budgets are untouched by the choice)."""
    from scopyon_gb300.base import _psf_for
    from scopyon_gb300.epifm import EngineConfig, FrameGraph, FramePipeline
    cfg = sg.DefaultConfiguration()
    upd = {"magnification": 100,
           "detector": {"type": det, "image_size": [96, 72], "exposure_time": 0.004},
           "effects": {"photo_bleaching": {"switch": True, "half_life": 0.02}}}
    if cmos_noise:
        upd["gpu"] = {"cmos_noise": cmos_noise}
        upd["analog_to_digital_converter"] = {"bit": 12, "offset": 100, "type": "pixel",
                                              "count": 5.0}
    cfg.update({"default": upd})
    t = numpy.arange(3 * 4 + 1) * 1e-3
    # reflecting walls keep the depths within the keys built below
    traj = sg.sample_inputs(t, N=800, lower=[-8e-6, -6e-6, -0.2e-6], upper=[8e-6, 6e-6, 0.2e-6],
                            D=0.4e-12, ndim=3, rng=numpy.random.RandomState(31),
                            boundary="reflecting")
    out = []
    for fused in (True, False):
        eng = EngineConfig(cfg["default"], rng=numpy.random.RandomState(4))
        pipe = FramePipeline(eng, "cuda", psf=_psf_for(eng, torch.device("cuda")))
        if pipe.camera_kind == 3:  # sCMOS: a per-pixel sigma map
            pipe.scmos_sigma_map(numpy.random.RandomState(5))
        pipe.psf.ensure(list(range(0, 202)))
        pipe.merge_camera = fused
        pipe.ensure_slots(800)
        pipe.budget[:800].copy_(torch.from_numpy(
            numpy.random.RandomState(6).exponential(0.02, 800) * eng.n_emit0))
        fg = FrameGraph(pipe, traj.copy(), 4, 1e-3, seed=9, use_graph=False)
        frames = []
        for _ in range(3):
            fg.step()
            frames.append((pipe.expect.cpu().numpy().copy(), pipe.adc32.cpu().numpy().copy()))
        pipe.check_status()
        out.append((frames, pipe.budget[:800].cpu().numpy().copy()))
    (f1, b1), (f0, b0) = out
    for (e1, a1), (e0, a0) in zip(f1, f0):
        numpy.testing.assert_array_equal(e1, e0)
        numpy.testing.assert_array_equal(a1, a0)
    numpy.testing.assert_array_equal(b1, b0)
    assert f1[0][0].max() > 0 and len(numpy.unique(f1[0][1])) > 10
