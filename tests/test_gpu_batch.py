"""GPU: batched fields of view packed into one canvas.

A small batch of fields with different sizes, emitter counts and diffusion
coefficients runs through one canvas frame.  Each field's expected image
must equal (1e-5 relative) the plain single-field pipeline fed with the same
trajectories in the field's own coordinates, and, for sampled fields, the
FP64 oracle's footprint sums; every emitter stays inside its field's walls.
"""

import math

import numpy
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sg():
    from scopyon_gb300 import _build
    _build.build()
    import scopyon_gb300
    return scopyon_gb300


def config1(sg, exposure=3e-3):
    """The single-channel TIRF / EMCCD configuration (EGFP, 160 nm pixels)."""
    cfg = sg.DefaultConfiguration()
    cfg.update({"default": {
        "magnification": 100,
        "fluorophore": {"type": "EGFP"},
        "detector": {"type": "EMCCD", "exposure_time": exposure, "QE": 0.92, "emgain": 300,
                     "readout_noise": 100},
        "analog_to_digital_converter": {"bit": 16, "offset": 2000, "fullwell": 800000},
        "light_source": {"flux_density": 1.1745e7},
        "effects": {"photo_bleaching": {"switch": False}}}})
    return cfg


def test_batched_fields_match_single_field_pipelines(sg):
    from scopyon_gb300.base import _psf_for
    from scopyon_gb300.batch import BatchedFields
    from scopyon_gb300.epifm import EngineConfig, FramePipeline
    import oracle as O
    sizes = [48, 64, 40, 96, 56, 64]
    counts = [30, 1, 120, 400, 0, 75]
    D = [1e-15, 1e-12, 3e-13, 5e-14, 1e-13, 1e-12]
    substeps = 5
    cfg = config1(sg)
    bf = BatchedFields(cfg, sizes, counts, D, frames=3, substeps=substeps, seed=3)
    bf.graph.use_graph = False
    for _ in range(2):
        bf.step()
    torch.cuda.synchronize()
    bf.pipe.check_status()
    canvas_expect = [bf.field_image(k, "expect").double().cpu().numpy() for k in range(len(sizes))]

    # the same trajectories: replay frame 1 (time indices substeps .. 2 substeps - 1)
    traj = bf.traj.copy()
    part = torch.empty(substeps * bf.n_emit * 5, dtype=torch.float64, device="cuda")
    traj.run(substeps, substeps, part)
    part = part.view(substeps, bf.n_emit, 5).cpu().numpy()
    W, H = bf.canvas
    px = bf.eng.px
    uts = numpy.full(substeps, bf.dt)
    start = numpy.cumsum([0] + counts)
    for k, s in enumerate(sizes):
        sl = slice(start[k], start[k + 1])
        i0, j0 = bf.origins[k]
        p = part[:, sl].copy()
        # every emitter is inside its field's walls
        assert ((p[..., 1] >= i0 * px - W * px / 2 - 1e-15) &
                (p[..., 1] <= (i0 + s) * px - W * px / 2 + 1e-15)).all()
        # field coordinates: relative to the field's centre
        p[..., 1] -= (i0 + s / 2) * px - W * px / 2
        p[..., 2] -= (j0 + s / 2) * px - H * px / 2
        p[..., 3] = numpy.arange(counts[k])
        fcfg = config1(sg)
        fcfg.update({"default": {"detector": {"image_size": [s, s]}}})
        eng = EngineConfig(fcfg["default"])
        pipe = FramePipeline(eng, "cuda", psf=_psf_for(eng, torch.device("cuda")))
        pipe.ensure_slots(max(counts[k], 1))
        if counts[k]:
            pipe.psf.ensure([0])
            expect, _, _ = pipe.run_frame(p, uts, with_optinfo=False, seed=1, counter=0)
            single = expect.double().cpu().numpy().reshape(s, s)
        else:  # no emitters: the background alone, QE * mean
            single = numpy.full((s, s), eng.qe * (eng.background_mean if eng.background_switch
                                                  else 0.0))
        ref = numpy.abs(single).max() + 1e-30
        assert numpy.abs(canvas_expect[k] - single).max() <= 1e-5 * ref, k
        if k in (0, 1) and counts[k]:
            # the FP64 oracle's footprint sums for the same emitters
            from scopyon_gb300.physics import emit_photons
            psf = O.PSFCache("EGFP", eng.psf_wavelength, None, eng.na, eng.radial_cutoff,
                             eng.depth_cutoff)
            n_emit = emit_photons(eng.amplitude0, bf.dt, eng.x_sec, eng.qy, eng.beer)
            norm = eng.norm_coeff * (1.0 * n_emit / (4.0 * numpy.pi))
            oracle = numpy.zeros((s, s))
            for st in range(substeps):
                for q in p[st]:
                    O.overlay_signal(oracle, psf.get(0.0), q[:3], px, norm)
            # the expectation is QE * (photons + background), _epifm.py:1430-1450
            bg = eng.background_mean if eng.background_switch else 0.0
            oracle = eng.qe * (oracle + bg)
            assert numpy.abs(canvas_expect[k] - oracle).max() <= 1e-5 * numpy.abs(oracle).max()


def test_autotune_and_graph_replay(sg):
    from scopyon_gb300.batch import BatchedFields
    rng = numpy.random.RandomState(1)
    sizes = list(rng.choice([32, 64, 128], 12))
    counts = list(numpy.exp(rng.uniform(math.log(10), math.log(2000), 12)).astype(int))
    D = list(numpy.exp(rng.uniform(math.log(1e-15), math.log(1e-12), 12)))
    bf = BatchedFields(config1(sg), sizes, counts, D, frames=24, substeps=4, seed=5)
    times = bf.autotune(frames=1)
    assert times and bf.tuning["chosen"]
    for _ in range(3):
        bf.step()
    torch.cuda.synchronize()
    bf.pipe.check_status()
    img = bf.field_image(3)
    assert img.shape == (sizes[3], sizes[3]) and torch.isfinite(img).all()


def test_pipelined_steps_match_single_frames(sg):
    """Two canvas frames per step (the second frame's records beside the first
    frame's splat) leave the same frame and trajectories as single steps."""
    from scopyon_gb300.batch import BatchedFields
    sizes, counts, D = [64, 48, 96], [50, 300, 20], [1e-13, 1e-12, 5e-14]
    out = []
    for per_step in (1, 2):
        bf = BatchedFields(config1(sg), sizes, counts, D, frames=8, substeps=4, seed=9,
                           frames_per_step=per_step)
        for _ in range(4 // per_step):
            bf.step()
        torch.cuda.synchronize()
        bf.pipe.check_status()
        out.append(([bf.field_image(k).clone() for k in range(3)], bf.traj._pos.clone()))
    for a, b in zip(out[0][0], out[1][0]):
        assert torch.equal(a, b)
    assert torch.equal(out[0][1], out[1][1])


def test_dense_field_accumulation_within_1e5_of_fp64(sg):
    """A bright field: 2000 emitters x 5 sub-steps on 24 x 24 px (about 3000
    footprint contributions per pixel) through the plain pipeline, against the
    FP64 oracle's footprint sums: the FP32 per-warp tile accumulation stays
    within 1e-5 relative per pixel."""
    from scopyon_gb300.base import _psf_for
    from scopyon_gb300.epifm import EngineConfig, FramePipeline
    from scopyon_gb300.physics import emit_photons
    import oracle as O
    cfg = config1(sg)
    cfg.update({"default": {"detector": {"image_size": [24, 24]},
                            "background": {"switch": False}}})
    eng = EngineConfig(cfg["default"])
    pipe = FramePipeline(eng, "cuda", psf=_psf_for(eng, torch.device("cuda")))
    rng = numpy.random.RandomState(21)
    n, substeps = 2000, 5
    half = 12 * eng.px
    part = numpy.zeros((substeps, n, 5))
    part[..., 1] = rng.uniform(-half, half, (substeps, n))
    part[..., 2] = rng.uniform(-half, half, (substeps, n))
    part[..., 3] = numpy.arange(n)
    part[..., 4] = 1.0
    pipe.ensure_slots(n)
    pipe.psf.ensure([0])
    dt = eng.exposure_time / substeps
    uts = numpy.full(substeps, dt)
    expect, _, _ = pipe.run_frame(part, uts, with_optinfo=False, seed=1, counter=0)
    got = expect.double().cpu().numpy().reshape(24, 24)
    psf = O.PSFCache("EGFP", eng.psf_wavelength, None, eng.na, eng.radial_cutoff, eng.depth_cutoff)
    n_emit = emit_photons(eng.amplitude0, dt, eng.x_sec, eng.qy, eng.beer)
    norm = eng.norm_coeff * (1.0 * n_emit / (4.0 * numpy.pi))
    ref = numpy.zeros((24, 24))
    for s in range(substeps):
        for q in part[s]:
            O.overlay_signal(ref, psf.get(0.0), q[:3], eng.px, norm)
    ref = eng.qe * ref
    rel = numpy.abs(got - ref).max() / numpy.abs(ref).max()
    assert rel <= 1e-5, rel


def _batch_pair(sg, fps, **kw):
    from scopyon_gb300.batch import BatchedFields
    sizes = [128, 256, 128, 512, 128, 256]
    counts = [4000, 20, 0, 30000, 900, 7000]
    D = [1e-15, 1e-12, 3e-13, 5e-14, 1e-13, 1e-12]
    cfg = config1(sg)
    out = []
    for persistent in (False, True):
        bf = BatchedFields(cfg, sizes, counts, D, frames=12, substeps=5, seed=8,
                           frames_per_step=fps, persistent=persistent, **kw)
        bf.pipe.set_tiles(16, 4, 4)
        out.append(bf)
    return out


@pytest.mark.parametrize("fps,graph", [(1, False), (2, True)])
def test_persistent_batch_frame_equals_canvas_form(sg, fps, graph):
    """The persistent launch (work list over tiles and camera chunks, bounded
    waits for each field's tiles) gives every field's expectation and ADC
    counts bit for bit as the canvas form (splat, merge, camera launches)."""
    canvas, persistent = _batch_pair(sg, fps)
    for bf in (canvas, persistent):
        bf.graph.use_graph = graph
    for step in range(3):
        canvas.step()
        persistent.step()
        torch.cuda.synchronize()
        canvas.pipe.check_status()
        persistent.pipe.check_status()
        for k in range(len(canvas.sizes)):
            for what in ("expect", "adc"):
                a = canvas.field_image(k, what).cpu().numpy()
                b = persistent.field_image(k, what).cpu().numpy()
                numpy.testing.assert_array_equal(a, b, err_msg="field %d %s step %d" % (k, what,
                                                                                         step))
    assert persistent.field_image(3, "expect").sum() > 0


def test_persistent_batch_wait_runs_out_and_is_reported(sg):
    """With a field tile count that no tile can reach (test hook) every
    chunk's bounded wait runs out: status bit 5, SC_ERR_TIMEOUT on the host,
    and the launch stops; with the hook off the next frame is correct."""
    from scopyon_gb300 import _lib
    canvas, persistent = _batch_pair(sg, 1)
    for bf in (canvas, persistent):
        bf.graph.use_graph = False
    persistent.target_extra, persistent.spin_limit = 1, 200
    persistent.step()
    torch.cuda.synchronize()
    assert persistent.pipe.status.cpu().numpy()[0] & 32
    with pytest.raises(_lib.ScopyonGPUError) as err:
        persistent.pipe.check_status()
    assert err.value.code == _lib.SC_ERR_TIMEOUT
    persistent.target_extra, persistent.spin_limit = 0, 0
    canvas.step()
    canvas.step()
    persistent.step()
    torch.cuda.synchronize()
    canvas.pipe.check_status()
    persistent.pipe.check_status()
    for k in range(len(canvas.sizes)):
        numpy.testing.assert_array_equal(canvas.field_image(k, "adc").cpu().numpy(),
                                         persistent.field_image(k, "adc").cpu().numpy())
