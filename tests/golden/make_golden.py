"""Generate golden vectors by running the reference scopyon itself.

Run here, where the reference source is mounted read-only:

    python tests/golden/make_golden.py /root/reference/src

It imports the reference package from that directory with four shims (pint,
``scopyon.constants``, ``scopyon.analysis`` and ``numpy.in1d`` are absent or
removed in this environment), passes configurations as SI dicts (PyYAML and
pint are absent), records every random draw the reference makes, and writes
``.npz`` fixtures next to this file.  The fixtures pin the oracle
(``tests/test_oracle_golden.py``) and feed the GPU parity tests, which never
read the reference at run time.
"""

import json
import os
import sys
import types

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def import_reference(src_dir):
    sys.dont_write_bytecode = True
    pint = types.ModuleType("pint")

    class _Quantity:
        pass

    pint.Quantity = _Quantity
    pint.UnitRegistry = lambda: None
    sys.modules["pint"] = pint
    const = types.ModuleType("scopyon.constants")
    const.N_A = 6.02214076e23
    const.hc = 6.62607015e-34 * 299792458
    const.Q_ = const.Quantity = _Quantity
    sys.modules["scopyon.constants"] = const
    sys.modules["scopyon.analysis"] = types.ModuleType("scopyon.analysis")
    if not hasattr(numpy, "in1d"):
        numpy.in1d = lambda a, b: numpy.isin(numpy.ravel(a), b)
    sys.path.insert(0, src_dir)
    import scopyon  # noqa: E402
    return scopyon


class RecordingRNG:
    """Wraps a RandomState and logs every draw the reference makes, in order."""

    def __init__(self, seed):
        self.r = numpy.random.RandomState(seed)
        self.log = []

    def normal(self, loc=0.0, scale=1.0, size=None):
        v = self.r.normal(loc, scale, size)
        self.log.append(("normal", numpy.array(v, dtype=float)))
        return v

    def uniform(self, low=0.0, high=1.0, size=None):
        v = self.r.uniform(low, high, size)
        self.log.append(("uniform", numpy.array(v, dtype=float)))
        return v

    def exponential(self, scale=1.0, size=None):
        v = self.r.exponential(scale, size)
        self.log.append(("exponential", numpy.array(v, dtype=float)))
        return v

    def poisson(self, lam=1.0, size=None):
        v = self.r.poisson(lam, size)
        self.log.append(("poisson", numpy.array(v, dtype=float)))
        return v

    def random_sample(self, size=None):
        v = self.r.random_sample(size)
        self.log.append(("random_sample", numpy.array(v, dtype=float)))
        return v

    def choice(self, a, size=None, replace=True, p=None):
        state = self.r.get_state()
        v = self.r.choice(a, size, replace, p)
        replay = numpy.random.RandomState()
        replay.set_state(state)
        self.log.append(("choice", numpy.array(replay.random_sample(), dtype=float)))
        return v


def si_tree(tree):
    """Replace ``{value, units}`` leaves by SI magnitudes (what pint would return)."""
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


def default_tree(**updates):
    sys.path.insert(0, ROOT)
    from scopyon_gb300.config import DefaultConfiguration
    cfg = DefaultConfiguration()
    cfg.update(updates)
    tree = si_tree(cfg.yaml)
    tree["default"].pop("gpu", None)
    return tree


def psf_goldens(scopyon, out):
    from scopyon._epifm import PointSpreadingFunction as PSF
    radial = numpy.arange(0.0, 1000e-9, 1e-9)
    depths = [0.0, 1e-9, 37e-9, 250.4e-9, 999e-9, 999.7e-9, 1000.5e-9, 1500e-9]
    for name, wl in (("tritc", 5.78e-07), ("egfp", 5.08e-07)):
        psf = PSF(1000e-9, None, 1000e-9, "Tetramethylrhodamine(TRITC)", wl)
        tabs, keys = [], []
        for d in depths:
            psf.get(d)
            key = [k for k in psf._PointSpreadingFunction__fluorophore_psf.keys()][-1]
            keys.append(key)
            dval = 1000e-9 if key == -1 else key * 1e-9
            tabs.append(psf.get_distribution(radial, dval))
        out["psf_%s_radial" % name] = numpy.array(tabs)
        out["psf_%s_keys" % name] = numpy.array(keys)
    out["psf_depths"] = numpy.array(depths)
    g = PSF(1000e-9, 1.0e-7, 1000e-9, "Gaussian", 6.0e-7)
    out["psf_gauss100_radial"] = g.get_distribution(radial, 0.0)

    psf = PSF(1000e-9, None, 1000e-9, "Tetramethylrhodamine(TRITC)", 5.78e-07)
    cart = psf.radial_to_cartesian(radial, out["psf_tritc_radial"][0], 1000e-9, 1e-9)
    out["cart_samples_idx"] = numpy.array([[999, 999], [0, 0], [999, 0], [0, 1998], [1500, 700],
                                           [1003, 995], [1998, 1998]])
    out["cart_samples"] = cart[tuple(out["cart_samples_idx"].T)]
    out["cart_total"] = cart.sum()

    cases = [
        ("c40_px160", (40, 40), 16e-6 / 100, [(0.0, 0.0), (3.3e-9, -7.77e-9), (1.23456789e-6, -2.2e-6),
                                              (3.1e-6, 3.15e-6), (5e-6, 0.0), (4.8e-7, -8.0e-7),
                                              (-3.2e-6, 2.9e-6)]),
        ("c96x64_px66", (96, 64), 16e-6 / 241, [(0.0, 0.0), (1.111e-6, -0.333e-6), (-3.1e-6, 2.05e-6)]),
    ]
    for depth_idx, tab in ((0, cart), (3, psf.radial_to_cartesian(
            radial, out["psf_tritc_radial"][3], 1000e-9, 1e-9))):
        for name, shape, px, positions in cases:
            imgs = []
            for (x, y) in positions:
                img = numpy.zeros(shape)
                PSF.overlay_signal_(img, tab, numpy.array([0.0, x, y]), px, 1e-9, 1.0)
                imgs.append(img)
            out["ov_%s_d%d" % (name, depth_idx)] = numpy.array(imgs)
            out["ov_%s_pos" % name] = numpy.array(positions)
            out["ov_%s_px" % name] = px
    img = numpy.zeros((512, 512))
    PSF.overlay_signal_(img, cart, numpy.zeros(3), 4.444444444444444e-08, 1e-9, 1.0)
    nz = numpy.nonzero(img)
    lo = (nz[0].min(), nz[1].min())
    hi = (nz[0].max() + 1, nz[1].max() + 1)
    out["ov_512_px44_window"] = numpy.array([lo[0], hi[0], lo[1], hi[1]])
    out["ov_512_px44"] = img[lo[0]:hi[0], lo[1]:hi[1]]


def physics_goldens(scopyon, out):
    from scopyon._epifm import EPIFMConfigs, _EPIFMSimulator
    rows = []
    for angle in (1.2566370614359172, 0.0, 1.1):
        tree = default_tree(default={"light_source": {"angle": angle}})
        configs = EPIFMConfigs(scopyon.Configuration(yaml=tree)["default"],
                               rng=numpy.random.RandomState(0))
        sim = _EPIFMSimulator(configs)
        amp, pen = sim.snells_law()
        n1 = _EPIFMSimulator.get_emit_photons(amp, 1.0, 83400, 0.61, 20e-9)
        n2 = _EPIFMSimulator.get_emit_photons(amp * 0.37, 3e-3, 56000, 0.6, 2.0e-9)
        rows.append([angle, amp, pen, n1, n2])
    out["physics_rows"] = numpy.array(rows)
    for fl in ("Tetramethylrhodamine(TRITC)", "EGFP"):
        tree = default_tree(default={"fluorophore": {"type": fl}})
        configs = EPIFMConfigs(scopyon.Configuration(yaml=tree)["default"],
                               rng=numpy.random.RandomState(0))
        tag = "tritc" if "TRITC" in fl else "egfp"
        out["cat_%s_psf_wavelength" % tag] = configs.psf_wavelength
        out["cat_%s_fluoem_norm_sum" % tag] = numpy.sum(configs.fluoem_norm)
    rn = numpy.loadtxt(os.path.join(scopyon.__path__[0], "catalog/detector/RNDist_F40.csv"),
                       delimiter=",")
    out["cmos_table"] = rn


def emccd_goldens(scopyon, out):
    from scopyon._epifm import EMCCD
    rows = []
    for e in (0.01, 0.5, 1.0, 3.7, 10.0, 55.0, 100.0, 333.3, 700.0):
        for seed in range(6):
            u = numpy.random.RandomState(seed).random_sample()
            sig = EMCCD.draw_signal(e, 300, numpy.random.RandomState(seed))
            rows.append([e, 300, u, sig])
        s, p = EMCCD.probability_distribution(e, 300)
        out["emccd_pdf_%g" % e] = numpy.stack([s.astype(float), p])
    out["emccd_draws"] = numpy.array(rows)


def adc_goldens(scopyon, out):
    from scopyon._epifm import EPIFMConfigs
    for fpn, count in (("none", 0.0), ("pixel", 5.0), ("column", 3.0)):
        tree = default_tree(default={
            "detector": {"image_size": [6, 5]},
            "analog_to_digital_converter": {"type": fpn, "count": count, "offset": 100,
                                            "bit": 12}})
        rng = RecordingRNG(11)
        configs = EPIFMConfigs(scopyon.Configuration(yaml=tree)["default"], rng=rng)
        out["adc_%s_offset" % fpn] = numpy.asarray(configs.ADConverter_offset, float)
        out["adc_%s_gain" % fpn] = numpy.asarray(configs.ADConverter_gain, float)
        out["adc_%s_normals" % fpn] = (rng.log[0][1] if rng.log else numpy.zeros(0))


def sampling_goldens(scopyon, out):
    t = numpy.arange(7) * 0.5e-3
    rng = numpy.random.RandomState(5)
    inp = scopyon.sample_inputs(t, N=5, lower=[-1e-6, -2e-6, -0.5e-6], upper=[1e-6, 2e-6, 0.5e-6],
                                D=0.1e-12, ndim=3, rng=rng)
    out["samp3_t"] = numpy.array([x for x, _ in inp])
    out["samp3_pts"] = numpy.array([p for _, p in inp])
    rng = numpy.random.RandomState(9)
    inp = scopyon.sample_inputs(t[:4], N=4, lower=-3e-6, upper=3e-6, D=[0.2e-12, 0.05e-12],
                                ndim=2, rng=rng)
    out["samp2_pts"] = numpy.array([p for _, p in inp])


def _frame_case(scopyon, out, name, tree, inputs, num_frames, seed, form=False,
                start_time=0.0, exposure_time=None):
    cfg = scopyon.Configuration(yaml=tree)
    rng = RecordingRNG(seed)
    sim = scopyon.EPIFMSimulator(cfg, method="default", rng=rng)
    frames, marks = [], [0]
    if form:
        img, info = sim.form_image(inputs, start_time, exposure_time, full_output=True)
        frames.append((img.as_array(), info))
        marks.append(len(rng.log))
    else:
        for img, info in sim.generate_images(inputs, num_frames, start_time, exposure_time,
                                             full_output=True):
            frames.append((img.as_array(), info))
            marks.append(len(rng.log))
    out["%s_config" % name] = json.dumps(tree)
    out["%s_adc" % name] = numpy.array([f[0] for f in frames])
    out["%s_expectation" % name] = numpy.array([f[1]["expectation"] for f in frames])
    ids = sorted(frames[0][1]["true_data"].keys())
    out["%s_true_ids" % name] = numpy.array(ids)
    out["%s_true_data" % name] = numpy.array(
        [[f[1]["true_data"][m] for m in ids] for f in frames])
    if "fluorescence_states" in frames[-1][1]:
        out["%s_states" % name] = numpy.array(
            [[f[1]["fluorescence_states"][m] for m in ids] for f in frames])
    # split the draw log: FPN normals at set-up, then per frame
    log = rng.log
    det = tree["default"]["detector"]["type"]
    fpn = tree["default"]["analog_to_digital_converter"]["type"]
    pos = 0
    if fpn != "none":
        out["%s_fpn_normals" % name] = log[0][1]
        pos = 1
    bleach = []
    for f in range(len(frames)):
        entries = log[max(marks[f], pos):marks[f + 1]]
        expected = frames[f][1]["expectation"]
        shape = expected.shape
        bl = [float(v) for k, v in entries if k == "exponential"]
        bleach.extend(bl)
        rest = [(k, v) for k, v in entries if k != "exponential"]
        if det == "EMCCD":
            noise = rest[0][1] if rest and rest[0][0] == "normal" else numpy.zeros(shape)
            us = [float(v) for k, v in rest if k == "choice"]
            uni = numpy.full(shape, numpy.nan).ravel()
            uni[expected.ravel() > 0] = us
            out["%s_f%d_noise" % (name, f)] = noise
            out["%s_f%d_uniform" % (name, f)] = uni.reshape(shape)
        elif det == "CCD":
            out["%s_f%d_noise" % (name, f)] = rest[0][1]
            out["%s_f%d_signal" % (name, f)] = numpy.array(
                [float(v) for k, v in rest if k == "poisson"]).reshape(shape)
        else:
            out["%s_f%d_uniform" % (name, f)] = numpy.array(
                [float(v) for k, v in rest if k == "choice"]).reshape(shape)
            out["%s_f%d_signal" % (name, f)] = numpy.array(
                [float(v) for k, v in rest if k == "poisson"]).reshape(shape)
    out["%s_bleach_times" % name] = numpy.array(bleach)
    if isinstance(inputs, numpy.ndarray):
        out["%s_inputs" % name] = inputs
    else:
        out["%s_input_t" % name] = numpy.array([t for t, _ in inputs])
        out["%s_input_pts" % name] = numpy.array([p for _, p in inputs])


def frame_goldens(scopyon, out):
    # (a) form_image, EMCCD, TIRF, 2-column inputs, peak pixels kept below ~700 e-
    rng = numpy.random.RandomState(123)
    px = 16e-6 / 100
    inputs = rng.uniform(-14 * px, 14 * px, size=(12, 2))
    inputs[0] = [0.0, 0.0]
    tree = default_tree(default={
        "magnification": 100, "fluorophore": {"type": "EGFP"},
        "detector": {"image_size": [32, 32], "exposure_time": 0.03},
        "light_source": {"flux_density": 1.0e6}})
    _frame_case(scopyon, out, "fa", tree, inputs, 1, 7, form=True)

    # (b) generate_images, CMOS table noise, EPI, 3-D trajectories, bleaching
    t = numpy.arange(0, 13) * 5e-3
    traj = scopyon.sample_inputs(t, N=9, lower=[-1.5e-6, -1.5e-6, -0.4e-6],
                                 upper=[1.5e-6, 1.5e-6, 0.4e-6], D=0.2e-12, ndim=3,
                                 rng=numpy.random.RandomState(3))
    tree = default_tree(default={
        "magnification": 100, "detector": {"type": "CMOS", "image_size": [24, 24],
                                           "exposure_time": 0.02},
        "light_source": {"angle": 0.0, "flux_density": 2.0e6},
        "analog_to_digital_converter": {"bit": 12, "offset": 100, "fullwell": 30000},
        "effects": {"photo_bleaching": {"switch": True, "half_life": 0.05}}})
    _frame_case(scopyon, out, "fb", tree, traj, 3, 21)

    # (c) CCD with per-pixel FPN, non-square image, 5-column inputs
    rng = numpy.random.RandomState(4)
    pts = numpy.hstack([rng.uniform(-1.2e-6, 1.2e-6, size=(6, 2)),
                        rng.uniform(-0.3e-6, 0.3e-6, size=(6, 1)),
                        numpy.arange(6)[:, None] + 10.0, numpy.ones((6, 1))])
    pts[2, 4] = 0.5
    tree = default_tree(default={
        "magnification": 100, "detector": {"type": "CCD", "image_size": [20, 16],
                                           "exposure_time": 0.01},
        "light_source": {"angle": 0.0},
        "analog_to_digital_converter": {"type": "pixel", "count": 4.0, "offset": 300}})
    _frame_case(scopyon, out, "fc", tree, [(0.0, pts)], 2, 5)

    # (d) EMCCD generate_images with Born-Wolf depth keys, TIRF, 2 frames x 3 sub-steps
    t = numpy.arange(0, 7) * 1e-3
    traj = scopyon.sample_inputs(t, N=5, lower=[-1.0e-6, -1.0e-6, 0.0],
                                 upper=[1.0e-6, 1.0e-6, 0.2e-6], D=0.5e-12, ndim=3,
                                 rng=numpy.random.RandomState(8))
    tree = default_tree(default={
        "magnification": 100, "fluorophore": {"type": "EGFP"},
        "detector": {"image_size": [20, 20], "exposure_time": 0.003},
        "light_source": {"flux_density": 3.0e6},
        "effects": {"photo_bleaching": {"switch": True, "half_life": 0.5}}})
    _frame_case(scopyon, out, "fd", tree, traj, 2, 13)


def main():
    src = sys.argv[1] if len(sys.argv) > 1 else "/root/reference/src"
    scopyon = import_reference(src)
    out = {}
    for fn in (psf_goldens, physics_goldens, emccd_goldens, adc_goldens, sampling_goldens,
               frame_goldens):
        fn(scopyon, out)
        print("done", fn.__name__, flush=True)
    out["versions"] = json.dumps({"numpy": numpy.__version__,
                                  "scipy": __import__("scipy").__version__,
                                  "python": sys.version.split()[0]})
    numpy.savez_compressed(os.path.join(HERE, "reference_goldens.npz"), **out)
    print("wrote", os.path.join(HERE, "reference_goldens.npz"))


if __name__ == "__main__":
    main()
