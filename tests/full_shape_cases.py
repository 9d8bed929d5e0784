"""Workloads at the benchmark configurations' own shapes, for parity tests.

config 1: plain TIRF, 1,000 emitters uniform over a 25.6 x 25.6 um field at
z = 0, D = 0.1 um^2/s, 30 ms frames in 10 sub-steps, EGFP, 160 nm pixels,
160 x 160 EMCCD (QE 0.92, gain 300, readout 100 e-, offset 2000, 16 bit),
100 photons per emitter per ms (flux density 1.1745e7 W/m^2).  The peak
pixels pass 709 e-, where the reference's EMCCD law overflows
(src/scopyon/_epifm.py:364-369); the oracle's log-shifted law does not.

config 2: EPI with defocus, emitters with x, y uniform over 512 x 512 pixels
and z uniform in [-1, 1] um, half at D = 0.01 and half at 1 um^2/s,
photobleaching with a 2 s mean lifetime, 10 ms frames in 20 sub-steps, TRITC,
CMOS with the reference's tabulated read noise and per-pixel offsets
rint N(100, 5), 12-bit ADC, fullwell 30,000 e-.

Inputs are seeded synthetic trajectories in the reference's host format
(``sample_inputs``: a list of ``(t, (N, k))`` arrays).
"""

import math

import numpy

import oracle as O

CFG1 = dict(n=1000, edge=160, substeps=10, exposure=0.030, D=0.1e-12)
CFG2 = dict(n=20000, edge=512, substeps=20, exposure=0.010, z_half=1e-6)


def si_tree(tree):
    """A configuration tree with ``{value, units}`` leaves in SI magnitudes."""
    from scopyon_gb300._units import to_base_magnitude
    out = {}
    for k, v in tree.items():
        if isinstance(v, dict):
            if "value" in v:
                out[k] = (to_base_magnitude(v["value"], v["units"])
                          if v["value"] is not None and "units" in v else v["value"])
            else:
                out[k] = si_tree(v)
        else:
            out[k] = v
    return out


def config1():
    import scopyon_gb300 as sg
    cfg = sg.DefaultConfiguration()
    cfg.update({"default": {
        "magnification": 100,
        "fluorophore": {"type": "EGFP"},
        "detector": {"type": "EMCCD", "image_size": [CFG1["edge"]] * 2,
                     "exposure_time": CFG1["exposure"], "QE": 0.92, "emgain": 300,
                     "readout_noise": 100},
        "analog_to_digital_converter": {"bit": 16, "offset": 2000, "fullwell": 800000,
                                        "type": "none"},
        "light_source": {"flux_density": 1.1745e7},
        "effects": {"photo_bleaching": {"switch": False}}}})
    return cfg


def config2(cmos_table, edge=None):
    import scopyon_gb300 as sg
    cfg = sg.DefaultConfiguration()
    cfg.update({"default": {
        "magnification": 100,
        "light_source": {"angle": 0.0},
        "detector": {"type": "CMOS", "image_size": [edge or CFG2["edge"]] * 2,
                     "exposure_time": CFG2["exposure"]},
        "analog_to_digital_converter": {"bit": 12, "offset": 100, "type": "pixel", "count": 5.0,
                                        "fullwell": 30000},
        "effects": {"photo_bleaching": {"switch": True, "half_life": 2.0 * math.log(2.0)}},
        "gpu": {"cmos_noise": "table", "cmos_table": numpy.asarray(cmos_table).tolist()}}})
    return cfg


def oracle_params(cfg, rng=None, cmos_table=None):
    """Oracle parameters of a configuration (catalog facts from the engine's lookup)."""
    import scopyon_gb300 as sg
    eng = sg.EPIFMSimulator(cfg, rng=numpy.random.RandomState(0)).base()
    tree = si_tree(cfg.yaml)["default"]
    return O.Params(tree, float(eng.psf_wavelength), eng.norm_coeff / eng.psf_normalization,
                    rng=rng, na=eng.na, cmos_table=cmos_table)


def inputs1(n_frames, seed=101):
    """config-1 trajectories: sample_inputs with ndim 2 -> (N, 4) [x, y, id, 1]."""
    c = CFG1
    t = numpy.arange(n_frames * c["substeps"] + 1) * (c["exposure"] / c["substeps"])
    half = c["edge"] * 160e-9 / 2
    return O.sample_inputs(t, c["n"], -half, half, c["D"], 2, numpy.random.RandomState(seed))


def inputs2(n_frames, n=None, seed=202, edge=None):
    """config-2 trajectories: (N, 5) [x, y, z, id, 1], two diffusion classes."""
    c = CFG2
    n = n or c["n"]
    edge = edge or c["edge"]
    rng = numpy.random.RandomState(seed)
    dt = c["exposure"] / c["substeps"]
    steps = n_frames * c["substeps"]
    half = edge * 160e-9 / 2
    pos = numpy.empty((steps + 1, n, 3))
    pos[0, :, 0] = rng.uniform(-half, half, n)
    pos[0, :, 1] = rng.uniform(-half, half, n)
    pos[0, :, 2] = rng.uniform(-c["z_half"], c["z_half"], n)
    d = numpy.where(numpy.arange(n) < n // 2, 0.01e-12, 1.0e-12)
    scale = numpy.sqrt(2 * d * dt)[:, None]
    for k in range(steps):
        pos[k + 1] = pos[k] + scale * rng.standard_normal((n, 3))
    ids = numpy.arange(n, dtype=float)[:, None]
    return [(k * dt, numpy.hstack([pos[k], ids, numpy.ones((n, 1))])) for k in range(steps + 1)]


def expectation_errors(e, e_ref, floor=1e-6):
    """(max relative error per pixel above floor * max, norm-wise relative error)."""
    big = e_ref > floor * e_ref.max()
    per_pixel = float((numpy.abs(e - e_ref)[big] / e_ref[big]).max())
    norm = float(numpy.abs(e - e_ref).sum() / e_ref.sum())
    return per_pixel, norm


def _emccd_chunk(job):
    e, u, g = job
    out = numpy.zeros(e.size)
    for i in range(e.size):
        if e[i] > 0:
            out[i] = O.emccd_draw(e[i], g, u[i])
    return out


def emccd_signal(expected, emgain, uniform, pool=None, workers=1):
    """The oracle's EMCCD inverse-CDF draws (_epifm.py:394-416) for a frame."""
    e, u = expected.ravel(), numpy.asarray(uniform).ravel()
    if pool is None or workers <= 1:
        return _emccd_chunk((e, u, emgain)).reshape(expected.shape)
    parts = numpy.array_split(numpy.arange(e.size), 4 * workers)
    res = pool.map(_emccd_chunk, [(e[p], u[p], emgain) for p in parts])
    return numpy.concatenate(res).reshape(expected.shape)
