"""FP64 numpy restatement of scopyon's image-formation path (test infrastructure).

Every function names the reference lines it restates; paths are relative to the
ecell/scopyon source tree (``src/scopyon/...``).  Floating-point operation order
follows the reference wherever it decides a discrete outcome (PSF depth keys,
pixel footprints, bleaching thresholds, inverse-CDF draws).
"""

import math

import numpy
import scipy.special

__all__ = [
    "N_A", "HC", "PSF_RES", "radial_grid", "born_wolf_radial", "gaussian_radial",
    "radial_to_cartesian", "psf_depth_key", "PSFCache", "footprints", "overlay_signal",
    "overlay_signal_sat", "quadrant_sat", "snells_law", "emit_photons", "photon_budget",
    "emccd_distribution", "emccd_draw", "adc_counts", "adc_maps", "Params", "NumpyDraws",
    "InjectedDraws", "output_frame", "generate_frames", "format_data", "sample_points",
    "move_points", "sample_inputs", "cmos_table_draw", "sampling2_sample",
]

# CODATA exact values; the reference derives the same numbers from pint
# (src/scopyon/constants.py:12-17).
N_A = 6.02214076e23
HC = 6.62607015e-34 * 299792458

# 1 nm radial and depth resolution of the PSF tables (src/scopyon/_epifm.py:61-62)
PSF_RES = 1e-9


# ----------------------------------------------------------------------------- PSF

def radial_grid(cutoff=1000.0e-9, res=PSF_RES):
    """Radii of the PSF table, ``arange(0, cutoff, res)`` (``_epifm.py:91``)."""
    return numpy.arange(0.0, cutoff, res, dtype=float)


def born_wolf_radial(r, depth, wavelength, na=1.4):
    """Born-Wolf defocus PSF, 100-term Riemann sum (``_epifm.py:181-213``).

    psf(r) = alpha^2/pi * |sum_k J0(r*alpha*rho_k) exp(-2i z gamma rho_k^2) rho_k drho|^2
    with rho_k = k/100, alpha = 2 pi NA / lambda, gamma = (2 pi / lambda) (NA/2)^2.
    """
    k = 2.0 * numpy.pi / wavelength
    alpha = k * na
    gamma = k * numpy.power(na / 2, 2)
    nterm = 100
    drho = 1.0 / nterm
    rho = numpy.arange(1, nterm + 1) * drho
    bessel = scipy.special.j0((numpy.asarray(r)[:, None] * alpha) * rho[None, :])
    phase = numpy.exp(-2 * 1.j * depth * gamma * rho * rho) * rho * drho
    total = (phase[None, :] * bessel).sum(axis=1)
    psf = numpy.abs(total) ** 2
    psf *= alpha * alpha / numpy.pi
    return psf


def gaussian_radial(r, sigma):
    """Gaussian PSF; depth is ignored (``_epifm.py:133-134``)."""
    return numpy.exp(-0.5 * (r / sigma) ** 2) / (2 * numpy.pi * sigma * sigma)


def _interp_linear(x, y, xq):
    """scipy ``interp1d(x, y)`` linear evaluation (searchsorted, clip, de Boor form)."""
    idx = numpy.searchsorted(x, xq).clip(1, len(x) - 1)
    x_lo, x_hi = x[idx - 1], x[idx]
    y_lo, y_hi = y[idx - 1], y[idx]
    return ((xq - x_lo) / (x_hi - x_lo)) * y_hi + ((x_hi - xq) / (x_hi - x_lo)) * y_lo


def radial_to_cartesian(radial, psf_r, res=PSF_RES):
    """(2n-1)^2 cartesian grid from a radial table, radius clamped (``_epifm.py:99-126``)."""
    n = radial.size
    offs = (numpy.arange(2 * n - 1) - (n - 1)) * res
    rr = numpy.sqrt(offs[None, :] ** 2 + offs[:, None] ** 2)
    rmax = radial.max()
    rr[rr > rmax] = rmax
    return _interp_linear(radial, psf_r, rr.ravel()).reshape(rr.shape)


def psf_depth_key(depth, cutoff_depth=1000.0e-9, res=PSF_RES):
    """1-nm depth key and the depth its table is built at (``_epifm.py:76-88``)."""
    depth = abs(depth)
    if depth < cutoff_depth + res:
        key = int(depth / res)
        return key, key * res
    return -1, cutoff_depth


class PSFCache:
    """Per-key cartesian PSF tables, built lazily like ``PointSpreadingFunction.get``."""

    def __init__(self, kind, wavelength=None, sigma=None, na=1.4,
                 radial_cutoff=1000.0e-9, depth_cutoff=1000.0e-9):
        self.kind, self.wavelength, self.sigma, self.na = kind, wavelength, sigma, na
        self.radial_cutoff, self.depth_cutoff = radial_cutoff, depth_cutoff
        self.tables, self.sats = {}, {}

    def radial(self, depth_value):
        r = radial_grid(self.radial_cutoff)
        if self.kind == "Gaussian":
            return gaussian_radial(r, self.sigma)
        return born_wolf_radial(r, depth_value, self.wavelength, self.na)

    def get(self, depth):
        key, depth_value = psf_depth_key(depth, self.depth_cutoff)
        if key not in self.tables:
            r = radial_grid(self.radial_cutoff)
            self.tables[key] = radial_to_cartesian(r, self.radial(depth_value))
        return self.tables[key]

    def get_sat(self, depth):
        key, _ = psf_depth_key(depth, self.depth_cutoff)
        if key not in self.sats:
            grid = self.get(depth)
            sat = numpy.zeros((grid.shape[0] + 1, grid.shape[1] + 1))
            sat[1:, 1:] = grid.cumsum(axis=0).cumsum(axis=1)
            self.sats[key] = sat
        return self.sats[key]


def footprints(n_pixel, pixel_length, coord, n_signal, res=PSF_RES):
    """Pixel indices and PSF-grid bounds along one axis (``_epifm.py:233-258``).

    Returns ``(pixels, bounds)``: pixel ``pixels[k]`` integrates grid rows
    ``bounds[k]:bounds[k+1]``.  ``None`` when the bound list is empty.
    """
    signal_width = res * (n_signal - 1)
    expected_width = n_pixel * pixel_length
    lo = math.floor((expected_width * 0.5 + coord - signal_width * 0.5) / pixel_length)
    hi = math.ceil((expected_width * 0.5 + coord + signal_width * 0.5) / pixel_length)
    pix = numpy.arange(max(0, lo), min(n_pixel, hi) + 1)
    bounds = (pix * pixel_length - (expected_width * 0.5 + coord - signal_width * 0.5)) / res
    bounds = numpy.ceil(bounds).astype(int)
    if len(bounds) == 0:
        return None
    bounds[0] = max(bounds[0], 0)
    bounds[-1] = min(bounds[-1], n_signal)
    return pix, bounds


def _slice_range(lo, hi, n):
    """Python slice semantics of ``signal[lo:hi]`` on an axis of length n."""
    lo, hi, _ = slice(lo, hi).indices(n)
    return lo, max(lo, hi)


def overlay_signal(expected, signal, p_i, pixel_length, normalization, res=PSF_RES):
    """Add one emitter's footprint sums to ``expected`` (``_epifm.py:224-282``)."""
    nw, nh = expected.shape
    fx = footprints(nw, pixel_length, p_i[1], signal.shape[0], res)
    if fx is None:
        return
    fy = footprints(nh, pixel_length, p_i[2], signal.shape[1], res)
    if fy is None:
        return
    (ix, bx), (jy, by) = fx, fy
    unit_area = res * res
    for k in range(len(bx) - 1):
        for m in range(len(by) - 1):
            photons = signal[bx[k]: bx[k + 1], by[m]: by[m + 1]].sum() * unit_area
            if photons > 0:
                expected[ix[k], jy[m]] += photons * normalization


def overlay_signal_sat(expected, sat, p_i, pixel_length, normalization, res=PSF_RES):
    """``overlay_signal`` evaluated from a summed-area table (same bounds, FP64)."""
    nw, nh = expected.shape
    ns0, ns1 = sat.shape[0] - 1, sat.shape[1] - 1
    fx = footprints(nw, pixel_length, p_i[1], ns0, res)
    if fx is None:
        return
    fy = footprints(nh, pixel_length, p_i[2], ns1, res)
    if fy is None:
        return
    (ix, bx), (jy, by) = fx, fy
    if len(bx) < 2 or len(by) < 2:
        return
    ax = numpy.array([_slice_range(bx[k], bx[k + 1], ns0) for k in range(len(bx) - 1)])
    ay = numpy.array([_slice_range(by[m], by[m + 1], ns1) for m in range(len(by) - 1)])
    a0, a1 = ax[:, 0][:, None], ax[:, 1][:, None]
    b0, b1 = ay[:, 0][None, :], ay[:, 1][None, :]
    block = sat[a1, b1] - sat[a0, b1] - sat[a1, b0] + sat[a0, b0]
    photons = block * (res * res)
    add = numpy.where(photons > 0, photons * normalization, 0.0)
    expected[numpy.ix_(ix[:-1], jy[:-1])] += add


def quadrant_sat(radial, psf_r, res=PSF_RES):
    """Exclusive 2-D prefix sum of one quadrant of the cartesian grid.

    ``G[u, v] = sum_{p<u, q<v} P[999+p, 999+q]`` for u, v in [0, n].  The full
    grid is symmetric about its centre in each axis, so any rectangle sum of
    it is a signed combination of ``G`` entries (the GPU table layout).
    """
    n = radial.size
    offs = numpy.arange(n) * res
    rr = numpy.sqrt(offs[None, :] ** 2 + offs[:, None] ** 2)
    rmax = radial.max()
    rr[rr > rmax] = rmax
    quad = _interp_linear(radial, psf_r, rr.ravel()).reshape(rr.shape)
    sat = numpy.zeros((n + 1, n + 1))
    sat[1:, 1:] = quad.cumsum(axis=0).cumsum(axis=1)
    return sat


# ------------------------------------------------------------------------ physics

def snells_law(flux_density, source_wavelength, angle):
    """Illumination amplitude and penetration depth (``_epifm.py:1362-1428``)."""
    n0 = flux_density / (HC / source_wavelength)
    sin2 = numpy.sin(angle) ** 2
    cos2 = numpy.cos(angle) ** 2
    n1, n2 = 1.46, 1.384
    r2 = (n2 / n1) ** 2
    if sin2 / r2 < 1:
        return n0, numpy.inf
    a2_x = n0 * (4 * cos2 * (sin2 - r2) / (r2 ** 2 * cos2 + sin2 - r2))
    a2_y = n0 * (4 * cos2 / (1 - r2))
    a2_z = n0 * (4 * cos2 * sin2 / (r2 ** 2 * cos2 + sin2 - r2))
    amplitude = ((a2_x + a2_z) + a2_y) / 2
    depth = source_wavelength / (4.0 * numpy.pi * numpy.sqrt(n1 ** 2 * sin2 - n2 ** 2))
    return amplitude, depth


def emit_photons(amplitude, unit_time, abs_coeff, qy, radius):
    """Photons emitted in ``unit_time`` (``_epifm.py:1344-1360``)."""
    x_sec = numpy.log(10) * abs_coeff * 0.1 / N_A
    n_abs = amplitude * x_sec * unit_time
    volume = (4.0 / 3.0) * numpy.pi * numpy.power(radius, 3)
    depth = 2.0 * radius
    a = (abs_coeff * 0.1 / N_A) * (1.0 / volume) * depth
    return qy * n_abs * (1.0 - numpy.power(10.0, -a))


def photon_budget(n_emit0, bleaching_time):
    """Budget from an Exp(half_life / ln 2) bleaching time (``_epifm.py:1487-1491``)."""
    return bleaching_time * n_emit0


# ------------------------------------------------------------------------- camera

def emccd_distribution(expected, emgain):
    """EMCCD output distribution over integer electrons (``_epifm.py:365-391``).

    Same support and weights as the reference; the exponent is shifted by its
    maximum before ``exp`` so that pixels above ~709 e- do not overflow (the
    shift cancels in the normalisation).
    """
    sigma = numpy.sqrt(expected) * 5 + 10
    s_min = max(0, emgain * int(expected - sigma))
    s_max = emgain * int(expected + sigma)
    s = numpy.arange(s_min, s_max)
    a = 1.0 / emgain
    x = a * s
    with numpy.errstate(divide="ignore", invalid="ignore"):
        y = 2 * numpy.sqrt(expected * x)
        expo = -x + y
        pos = s > 0
        shift = expo[pos].max() if pos.any() else 0.0
        p = numpy.zeros(s.shape)
        p[pos] = 1.0 / y[pos] * numpy.exp(expo[pos] - shift) * scipy.special.i1e(y[pos])
    if s[0] <= 0:
        p[0] = 1.0 / (2 * a * expected) * numpy.exp(-shift)
    p /= p.sum()
    return s, p


def emccd_draw(expected, emgain, uniform):
    """Inverse-CDF draw of ``numpy.random.RandomState.choice`` (``_epifm.py:394-400``)."""
    if expected <= 0:
        return 0
    s, p = emccd_distribution(expected, emgain)
    cdf = p.cumsum()
    cdf /= cdf[-1]
    return s[cdf.searchsorted(uniform, side="right")]


def cmos_table_draw(table, uniform):
    """Additive CMOS noise from the tabulated distribution (``_epifm.py:332-345``)."""
    prob = table[:, 1] / table[:, 1].sum()
    cdf = prob.cumsum()
    cdf /= cdf[-1]
    return table[cdf.searchsorted(uniform, side="right"), 0]


def adc_counts(photoelectron, fullwell, gain, offset, bit):
    """Analog-to-digital conversion, clipped, not rounded (``_epifm.py:1473-1484``)."""
    adc = numpy.array(photoelectron, dtype=float, copy=True)
    adc[adc > fullwell] = fullwell
    adc_max = 2 ** bit - 1
    adc /= gain
    adc += offset
    adc[adc > adc_max] = adc_max
    adc[adc < 0] = 0
    return adc


def adc_maps(nw, nh, bit, fullwell, offset0, fpn_type, fpn_count, rng=None):
    """Per-pixel ADC offset and gain maps (``_epifm.py:926-963``)."""
    if fpn_type == "none":
        offset = numpy.full(nw * nh, offset0)
    elif fpn_type == "pixel":
        offset = numpy.rint(rng.normal(offset0, fpn_count, nw * nh))
    elif fpn_type == "column":
        column = rng.normal(offset0, fpn_count, nh)
        offset = numpy.rint(numpy.tile(column, (1, nw)).reshape(nh * nw))
    else:
        raise ValueError("FPN type [%s] is invalid ['pixel', 'column' or 'none']" % fpn_type)
    gain = (fullwell - 0.0) / (pow(2.0, bit) - offset)
    return offset.reshape([nw, nh]), gain.reshape([nw, nh])


# ------------------------------------------------------------------ frame driver

class Params:
    """Numbers the frame driver needs, taken from an SI configuration tree.

    ``tree`` is the method sub-tree with SI magnitudes (what the reference's
    ``EPIFMConfigs.initialize`` reads, ``_epifm.py:762-797``).  The catalog
    lookups of ``set_fluorophore`` (``_epifm.py:822-869``) are passed in as
    ``psf_wavelength`` and ``fluoem_norm_sum``.
    """

    def __init__(self, tree, psf_wavelength, fluoem_norm_sum=1.0, rng=None, na=1.4,
                 cmos_table=None):
        fl, det, adc = tree["fluorophore"], tree["detector"], tree["analog_to_digital_converter"]
        src, eff = tree["light_source"], tree["effects"]
        self.fluorophore_type = fl["type"]
        self.radius = fl["radius"]
        self.psf_normalization = fl["normalization"]
        self.psf_wavelength = psf_wavelength
        self.fluoem_norm_sum = fluoem_norm_sum
        self.radial_width = fl.get("radial_width")
        self.radial_cutoff, self.depth_cutoff = fl["radial_cutoff"], fl["depth_cutoff"]
        self.flux_density, self.source_wavelength = src["flux_density"], src["wave_length"]
        self.angle = src["angle"]
        self.magnification = tree["magnification"]
        self.detector_type = det["type"]
        self.image_size = det["image_size"]
        self.pixel_length = det["pixel_length"]
        self.exposure_time = det["exposure_time"]
        self.focal_point = det["focal_point"]
        self.qe, self.readout_noise, self.emgain = det["QE"], det["readout_noise"], det["emgain"]
        self.bit, self.fullwell = adc["bit"], adc["fullwell"]
        sh = tree.get("shutter", {}) or {}
        self.shutter_switch = sh.get("switch", False)
        self.shutter_start, self.shutter_end = sh.get("start_time"), sh.get("end_time")
        self.background_switch = eff["background"]["switch"]
        self.background_mean = eff["background"]["mean"]
        self.qy = eff["fluorescence"]["quantum_yield"]
        self.abs_coeff = eff["fluorescence"]["abs_coefficient"]
        self.bleach_switch = eff["photo_bleaching"]["switch"]
        self.half_life = eff["photo_bleaching"]["half_life"]
        self.offset, self.gain = adc_maps(self.image_size[0], self.image_size[1], self.bit,
                                          self.fullwell, adc["offset"], adc["type"],
                                          adc["count"], rng)
        self.cmos_table = cmos_table
        self.psf = PSFCache(self.fluorophore_type, psf_wavelength, self.radial_width, na,
                            self.radial_cutoff, self.depth_cutoff)

    @property
    def px(self):
        return self.pixel_length / self.magnification


class NumpyDraws:
    """Draws taken from a ``numpy.random.RandomState`` in the reference's order."""

    def __init__(self, rng):
        self.rng = rng

    def bleaching_time(self, m_id, beta):
        return self.rng.exponential(scale=beta, size=None)

    def camera(self, params, expected):
        rng, shape = self.rng, expected.shape
        out = {}
        if params.detector_type == "CMOS":
            u = numpy.empty(shape)
            for i in range(shape[0]):
                for j in range(shape[1]):
                    u[i, j] = rng.random_sample()
            out["noise"] = cmos_table_draw_array(params.cmos_table, u)
            sig = numpy.empty(shape)
            for i in range(shape[0]):
                for j in range(shape[1]):
                    sig[i, j] = rng.poisson(expected[i, j], None)
            out["signal"] = sig
        elif params.detector_type in ("EMCCD", "CCD"):
            if params.readout_noise <= 0:
                out["noise"] = numpy.zeros(shape)
            else:
                out["noise"] = rng.normal(0, params.readout_noise, shape)
            if params.detector_type == "CCD":
                sig = numpy.empty(shape)
                for i in range(shape[0]):
                    for j in range(shape[1]):
                        sig[i, j] = rng.poisson(expected[i, j], None)
                out["signal"] = sig
            else:
                flat = expected.ravel()
                sig = numpy.zeros(flat.size)
                for i in range(flat.size):
                    if flat[i] > 0:
                        sig[i] = emccd_draw(flat[i], params.emgain, rng.random_sample())
                out["signal"] = sig.reshape(shape)
        else:
            raise RuntimeError("Unknown detector type was given [%s]." % params.detector_type)
        return out


def cmos_table_draw_array(table, uniform):
    prob = table[:, 1] / table[:, 1].sum()
    cdf = prob.cumsum()
    cdf /= cdf[-1]
    return table[cdf.searchsorted(uniform, side="right"), 0]


class InjectedDraws:
    """Draws supplied by the caller: recorded from a reference run, or synthetic.

    ``bleach``: {m_id: bleaching time}; ``frames``: list of dicts per frame with
    ``noise`` (electrons, W x H) and either ``signal`` (W x H electrons) or
    ``uniform`` (W x H, consumed by the EMCCD inverse CDF or the CMOS table).
    """

    def __init__(self, bleach=None, frames=None):
        self.bleach, self.frames, self.frame = bleach or {}, frames or [], 0

    def bleaching_time(self, m_id, beta):
        return self.bleach[m_id]

    def camera(self, params, expected):
        d = self.frames[self.frame]
        self.frame += 1
        out = {"noise": numpy.asarray(d["noise"], dtype=float)}
        if "signal" in d:
            out["signal"] = numpy.asarray(d["signal"], dtype=float)
        elif params.detector_type == "EMCCD":
            flat, u = expected.ravel(), numpy.asarray(d["uniform"]).ravel()
            sig = numpy.zeros(flat.size)
            for i in range(flat.size):
                if flat[i] > 0:
                    sig[i] = emccd_draw(flat[i], params.emgain, u[i])
            out["signal"] = sig.reshape(expected.shape)
        else:
            raise ValueError("injected draws need 'signal' for %s" % params.detector_type)
        if params.detector_type == "CMOS" and "noise" not in d:
            out["noise"] = cmos_table_draw_array(params.cmos_table, d["uniform"])
        return out


def output_frame(params, input_data, draws, frame_index=0, start_time=0.0,
                 exposure_time=None, states=None, use_sat=False):
    """One camera frame (``_epifm.py:1121-1225`` with ``:1267-1333``, ``:1430-1470``).

    ``input_data`` is the formatted list of ``(t, (N,5) [depth,x,y,m_id,p_state])``.
    Returns ``(camera (W,H,2), infodict)`` like the reference.
    """
    exposure_time = exposure_time or params.exposure_time
    times = numpy.array([t for t, _ in input_data])
    t = start_time + exposure_time * frame_index
    if params.shutter_switch:
        t = max(t, params.shutter_start)
        exposure_time = max(0.0, min(t + exposure_time, params.shutter_end))
    start = numpy.searchsorted(times, t, side="right")
    if start != 0:
        start -= 1
    stop = numpy.searchsorted(times, t + exposure_time, side="left")
    frame_data = input_data[start:stop]

    p_0 = numpy.asarray(params.focal_point)
    nw, nh = params.image_size
    px = params.px
    camera = numpy.zeros((nw, nh, 2))
    optinfo = {}
    amplitude0, penetration = snells_law(params.flux_density, params.source_wavelength,
                                         params.angle)
    n_emit0 = emit_photons(amplitude0, 1.0, params.abs_coeff, params.qy, params.radius)
    beta = params.half_life / numpy.log(2.0) if params.bleach_switch else None

    for i, (i_time, particles) in enumerate(frame_data):
        current = i_time if i != 0 else t
        nxt = frame_data[i + 1][0] if i + 1 < len(frame_data) else t + exposure_time
        unit_time = nxt - current
        if unit_time < 1e-13:
            continue
        expected = numpy.zeros((nw, nh))
        for particle in particles:
            x, y, z, m_id, p_state = particle
            m_id = int(m_id)
            p_i = numpy.array([x, y, z])
            rel = p_i - p_0
            depth = rel[0]
            amplitude = amplitude0 * numpy.exp(-abs(depth) / penetration)
            n_emit = emit_photons(amplitude, unit_time, params.abs_coeff, params.qy,
                                  params.radius)
            if states is not None and params.bleach_switch:
                if m_id not in states:
                    states[m_id] = photon_budget(n_emit0, draws.bleaching_time(m_id, beta))
                budget = states[m_id] - n_emit
                if budget <= 0:
                    budget = 0
                    p_state = 0.0
                states[m_id] = budget
            norm = params.fluoem_norm_sum * params.psf_normalization
            norm *= p_state * n_emit / (4.0 * numpy.pi)
            if norm > 0.0:
                if use_sat:
                    overlay_signal_sat(expected, params.psf.get_sat(depth), rel, px, norm)
                else:
                    overlay_signal(expected, params.psf.get(depth), rel, px, norm)
            if m_id not in optinfo:
                optinfo[m_id] = numpy.zeros(8)
            optinfo[m_id] += numpy.array([
                unit_time, unit_time * p_state, unit_time * p_i[1], unit_time * p_i[2],
                unit_time * p_i[1], unit_time * p_i[2], unit_time * depth, norm])
        camera[:, :, 0] += expected

    for m_id in optinfo:
        optinfo[m_id][1] /= exposure_time
        optinfo[m_id][2:6] /= optinfo[m_id][0]
        optinfo[m_id][2] = (optinfo[m_id][2] - p_0[1]) / px + (nw - 1) * 0.5
        optinfo[m_id][3] = (optinfo[m_id][3] - p_0[2]) / px + (nh - 1) * 0.5

    photons = camera[:, :, 0]
    if params.background_switch:
        photons += params.background_mean
    expected = params.qe * photons
    cam = draws.camera(params, expected)
    camera[:, :, 0] = expected
    camera[:, :, 1] = adc_counts(cam["signal"] + cam["noise"], params.fullwell, params.gain,
                                 params.offset, params.bit)
    info = dict(true_data=optinfo)
    if states is not None:
        info["fluorescence_states"] = dict(states)
    return camera, info


def generate_frames(params, input_data, num_frames, draws, start_time=0.0,
                    exposure_time=None, use_sat=False):
    """Frame generator with bleaching state carried over (``_epifm.py:1017-1049``)."""
    states = {} if params.bleach_switch else None
    exposure_time = exposure_time or params.exposure_time
    for f in range(num_frames):
        yield output_frame(params, input_data, draws, f, start_time, exposure_time, states,
                           use_sat)


# ------------------------------------------------------------------------ inputs

def format_data(inputs, scale=1.0, origin=(0.0, 0.0, 0.0), unit_x=(1.0, 0.0, 0.0),
                unit_y=(0.0, 1.0, 0.0)):
    """Columns to ``[depth, x, y, m_id, p_state]`` (``src/scopyon/base.py:61-110``)."""
    inputs = numpy.asarray(inputs)
    n, k = inputs.shape
    if k == 2:
        data = numpy.zeros((n, 5))
        data[:, 1:3] = inputs * scale
        data[:, 3] = numpy.arange(n)
        data[:, 4] = 1.0
    elif k in (3, 5):
        origin = numpy.array(origin)
        pos = inputs[:, :3] * scale - origin
        unit_z = numpy.cross(unit_x, unit_y)
        data = numpy.zeros((n, 5))
        data[:, 0] = numpy.dot(pos, unit_z)
        data[:, 1] = numpy.dot(pos, unit_x)
        data[:, 2] = numpy.dot(pos, unit_y)
        if k == 3:
            data[:, 3] = numpy.arange(n)
            data[:, 4] = 1.0
        else:
            data[:, 3:] = inputs[:, 3:]
    elif k == 4:
        data = numpy.zeros((n, 5))
        data[:, 1:3] = inputs[:, :2] * scale
        data[:, 3:] = inputs[:, 2:]
    else:
        raise ValueError("The given 'inputs' has wrong shape.")
    return data


def sample_points(rng, n, lower, upper, start=0, ndim=3):
    """Uniform initial points, column by column (``src/scopyon/sampling.py:14-86``)."""
    lower = numpy.ones(ndim) * lower if numpy.isscalar(lower) else numpy.array(lower, float)
    upper = numpy.ones(ndim) * upper if numpy.isscalar(upper) else numpy.array(upper, float)
    for d in range(ndim):
        if lower[d] > upper[d]:
            lower[d], upper[d] = upper[d], lower[d]
    out = numpy.zeros((n, ndim + 2))
    for d in range(ndim):
        out[:, d] = rng.uniform(lower[d], upper[d], n) if lower[d] < upper[d] else lower[d]
    out[:, ndim] = numpy.arange(start, start + n)
    out[:, ndim + 1] = 1.0
    return out


def move_points(normals, points, D, dt, ndim=3):
    """Brownian step with given standard normals (``src/scopyon/sampling.py:88-119``).

    ``normals`` has shape (N, ndim) and is consumed particle-major, axis-minor,
    which is the order of the reference's scalar ``rng.normal`` calls.
    """
    D = numpy.zeros(ndim) if D is None else (
        numpy.ones(ndim) * D if numpy.isscalar(D) else numpy.asarray(D, float))
    out = points.copy()
    scale = numpy.sqrt(2 * D * dt)
    out[:, :ndim] += scale[None, :] * normals
    return out


def sample_inputs(t, n, lower, upper, D, ndim, rng, start=0):
    """Time-stamped trajectories (``src/scopyon/sampling.py:121-162``)."""
    t = sorted(t)
    points = sample_points(rng, n, lower, upper, start, ndim)
    current = t[0]
    out = []
    for nxt in t:
        if nxt > current:
            points = move_points(rng.standard_normal((len(points), ndim)), points, D,
                                 nxt - current, ndim)
            current = nxt
        else:
            points = points.copy()
        out.append((current, points))
    return out


# ------------------------------------------------------- multi-state sampler
def sampling2_sample(t, N, lower, upper, D, transmat, ndim, periodic, rng):
    """Multi-state Brownian points (``src/scopyon/sampling2.py:15-68``, ``:70-148``).

    Returns one (n, ndim + 2) array [coords, state, id] per time point.  Draw
    order: initial points per state block and axis (``:15-31``); per time step
    with dt > 0, one normal per particle and axis, particle-major (``:33-50``),
    then, with a rate matrix, one uniform per particle (``:52-68``).  The
    transition uses searchsorted side 'left' (the reference writes 'leff').
    """
    N = list(N) if hasattr(N, "__iter__") else [N]
    lower = numpy.ones(ndim) * lower if numpy.isscalar(lower) else numpy.array(lower, float)
    upper = numpy.ones(ndim) * upper if numpy.isscalar(upper) else numpy.array(upper, float)
    for d in range(ndim):
        if lower[d] > upper[d]:
            lower[d], upper[d] = upper[d], lower[d]
    D = numpy.ones(len(N)) * D if numpy.isscalar(D) else numpy.asarray(D, float)
    pts = numpy.zeros((sum(N), ndim + 2))
    tot = 0
    for i, cnt in enumerate(N):
        for d in range(ndim):
            pts[tot:tot + cnt, d] = (rng.uniform(lower[d], upper[d], cnt) if lower[d] < upper[d]
                                     else lower[d])
        pts[tot:tot + cnt, ndim] = i
        tot += cnt
    pts[:, ndim + 1] = numpy.arange(pts.shape[0])
    out = [pts.copy()]
    current = t[0]
    for nxt in t[1:]:
        if nxt > current:
            dt = nxt - current
            state = pts[:, ndim].astype(int)
            scale = numpy.sqrt(2 * D[state] * dt)
            pts = pts.copy()
            pts[:, :ndim] += scale[:, None] * rng.standard_normal((pts.shape[0], ndim))
            if periodic:
                for d in range(ndim):
                    if upper[d] > lower[d]:
                        pts[:, d] = (pts[:, d] - lower[d]) % (upper[d] - lower[d]) + lower[d]
                    else:
                        pts[:, d] = lower[d]
            if transmat is not None:
                rates = numpy.asarray(transmat, float)
                n = rates.shape[0]
                P = 1 - numpy.exp(-rates * dt)
                P.ravel()[::n + 1] = 1.0 - P.sum(axis=1)
                Pacc = P.cumsum(axis=1)
                u = rng.uniform(0, 1, pts.shape[0])
                pts[:, ndim] = [numpy.searchsorted(Pacc[s], r, side="left")
                                for s, r in zip(state, u)]
            current = nxt
        out.append(pts)
    return out
