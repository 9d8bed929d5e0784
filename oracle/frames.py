"""Vectorised FP64 frames for many emitters (test infrastructure).

``output_frame`` in ``epifm.py`` follows the reference particle by particle
and builds a 1999 x 1999 grid per depth key, which is fine for the golden
frames (a dozen emitters) but not for a 512 x 512 frame with 20,000 emitters
over 20 sub-steps and a thousand depth keys.  This module computes the same
frame with the same FP64 decisions, vectorised over emitters:

* per-emitter physics and photobleaching (``_epifm.py:1267-1315``,
  ``:1344-1360``, ``:1487-1491``) over all particles of a sub-step at once;
* the footprint bounds of ``overlay_signal_`` (``_epifm.py:233-275``) for all
  records at once, with the same FP64 operations in the same order, so every
  ``ceil`` decides as the reference's does;
* the slice sums ``signal[i0:i1, j0:j1].sum()`` (``_epifm.py:277-282``) as
  differences of an exact FP64 prefix sum.  The cartesian grid is symmetric
  about its centre in both axes (``radial_to_cartesian``, ``_epifm.py:99-126``),
  so a prefix sum of the full grid is a signed sum of at most 3 x 3 entries of
  the prefix sum of one quadrant; only that quadrant (1001^2 entries) is built
  per depth key, and keys are processed one at a time (optionally by a pool of
  spawned worker processes), so memory stays small for any number of keys.

``tests/test_oracle_frames.py`` pins this module to ``epifm.output_frame``
(itself pinned to the reference's own frames) on shared inputs.
"""

import numpy

from .epifm import (PSF_RES, adc_counts, born_wolf_radial, emit_photons, gaussian_radial,
                    photon_budget, radial_grid, snells_law)

__all__ = ["QuadrantGeometry", "quadrant_prefix", "full_prefix_terms", "axis_footprints",
           "depth_keys", "splat_records", "frame_records", "splat_frame", "output_frame_fast"]


class QuadrantGeometry:
    """Interpolation indices and weights of one quadrant of the cartesian grid.

    ``radial_to_cartesian`` (``_epifm.py:99-126``) evaluates scipy's linear
    ``interp1d`` at R = sqrt(dx^2 + dy^2) (clamped to the table's last radius)
    for every grid point; R, the bracketing index and the two weights depend
    only on the geometry, so they are computed once here with the same FP64
    operations as ``epifm._interp_linear``.
    """

    def __init__(self, radial_cutoff=1000.0e-9, res=PSF_RES):
        self.r = radial_grid(radial_cutoff, res)
        n = self.r.size
        self.n = n
        offs = numpy.arange(n) * res
        rr = numpy.sqrt(offs[None, :] ** 2 + offs[:, None] ** 2)
        rmax = self.r.max()
        rr[rr > rmax] = rmax
        idx = numpy.searchsorted(self.r, rr.ravel()).clip(1, n - 1)
        x_lo, x_hi = self.r[idx - 1], self.r[idx]
        self.idx = idx
        self.w_hi = (rr.ravel() - x_lo) / (x_hi - x_lo)
        self.w_lo = (x_hi - rr.ravel()) / (x_hi - x_lo)


def quadrant_prefix(geom, psf_r):
    """G[u, v] = sum_{p < u, q < v} P[c + p, c + q], c = n - 1, u, v in [0, n].

    P is the full cartesian grid of the radial table ``psf_r``; the quadrant
    values equal ``radial_to_cartesian``'s bit for bit (same interpolation
    arithmetic), and the prefix sums are FP64 cumulative sums.
    """
    n = geom.n
    quad = (geom.w_hi * psf_r[geom.idx] + geom.w_lo * psf_r[geom.idx - 1]).reshape(n, n)
    g = numpy.zeros((n + 1, n + 1))
    g[1:, 1:] = quad.cumsum(axis=0).cumsum(axis=1)
    return g


def full_prefix_terms(bounds, n):
    """Signed quadrant-prefix terms of the full grid's prefix along one axis.

    For a full-grid bound g in [0, 2n - 1], sum_{g' < g} P[g'] with P[g'] =
    q[|g' - (n - 1)|] equals sum_i sign_i * Gq(u_i):
    g <= n - 1: Gq(n) - Gq(n - g);  g >= n - 1: Gq(n) - Gq(1) + Gq(g - n + 1).
    Returns (u, sign), each of shape bounds.shape + (3,).
    """
    b = numpy.asarray(bounds, dtype=numpy.int64)
    low = b <= n - 1
    u = numpy.empty(b.shape + (3,), dtype=numpy.int64)
    s = numpy.empty(b.shape + (3,))
    u[..., 0], s[..., 0] = n, 1.0
    u[..., 1] = numpy.where(low, n - b, 1)
    s[..., 1] = -1.0
    u[..., 2] = numpy.where(low, 0, b - n + 1)
    s[..., 2] = 1.0
    return u, s


def axis_footprints(n_pixel, pixel_length, coord, n_signal, res=PSF_RES, width=None):
    """``footprints`` (``_epifm.py:233-258``) for an array of coordinates.

    Returns (first pixel (R,), bound count (R,), bounds (R, width + 1)):
    pixel first + k integrates grid rows bounds[k]:bounds[k+1] for k < count - 1;
    bounds past the count repeat the last one.  FP64 operations and their order
    are the reference's, so every ceil and floor decides identically.
    """
    coord = numpy.asarray(coord, dtype=float)
    signal_width = res * (n_signal - 1)
    expected_width = n_pixel * pixel_length
    lo = numpy.floor((expected_width * 0.5 + coord - signal_width * 0.5) / pixel_length)
    hi = numpy.ceil((expected_width * 0.5 + coord + signal_width * 0.5) / pixel_length)
    first = numpy.maximum(0, lo).astype(numpy.int64)
    last = numpy.minimum(n_pixel, hi).astype(numpy.int64)
    count = numpy.maximum(last - first + 1, 0)
    if width is None:
        width = int(numpy.ceil(signal_width / pixel_length)) + 2
    if (count > width + 1).any():
        raise ValueError("footprint wider than the window")
    k = numpy.arange(width + 1)
    pix = first[:, None] + k[None, :]
    org = expected_width * 0.5 + coord - signal_width * 0.5
    bounds = numpy.ceil((pix * pixel_length - org[:, None]) / res).astype(numpy.int64)
    rows = numpy.arange(len(coord))
    has = count > 0
    bounds[rows[has], 0] = numpy.maximum(bounds[rows[has], 0], 0)
    lastk = numpy.clip(count - 1, 0, width)
    bounds[rows[has], lastk[has]] = numpy.minimum(bounds[rows[has], lastk[has]], n_signal)
    # bounds past the last repeat it (zero-width slices)
    past = k[None, :] > lastk[:, None]
    bounds = numpy.where(past, bounds[rows, lastk][:, None], bounds)
    return first, count, bounds


def splat_records(image, gq, n_r, x, y, norm, pixel_length, res=PSF_RES):
    """Add footprints of records sharing one depth key (``_epifm.py:224-282``).

    image: (nw, nh) FP64, updated in place.  gq: the key's quadrant prefix;
    x, y: the records' positions relative to the focal point (axis 0 of the
    image is x); norm: their normalisations.  A pixel receives
    (slice sum * res^2) * norm when the slice sum is positive.
    """
    nw, nh = image.shape
    n_signal = 2 * n_r - 1
    fx0, cx, bx = axis_footprints(nw, pixel_length, x, n_signal, res)
    fy0, cy, by = axis_footprints(nh, pixel_length, y, n_signal, res)
    ok = (cx >= 2) & (cy >= 2)
    if not ok.any():
        return
    fx0, cx, bx, fy0, cy, by, norm = fx0[ok], cx[ok], bx[ok], fy0[ok], cy[ok], by[ok], norm[ok]
    ux, sx = full_prefix_terms(bx, n_r)
    uy, sy = full_prefix_terms(by, n_r)
    # full-grid prefix at every (x bound, y bound) pair: 3 x 3 signed terms
    c2 = numpy.zeros((len(norm), bx.shape[1], by.shape[1]))
    for i in range(3):
        for j in range(3):
            c2 += (sx[:, :, None, i] * sy[:, None, :, j]) * gq[ux[:, :, None, i], uy[:, None, :, j]]
    block = c2[:, 1:, 1:] - c2[:, :-1, 1:] - c2[:, 1:, :-1] + c2[:, :-1, :-1]
    photons = block * (res * res)
    kx = numpy.arange(bx.shape[1] - 1)
    ky = numpy.arange(by.shape[1] - 1)
    valid = ((kx[None, :, None] < (cx - 1)[:, None, None])
             & (ky[None, None, :] < (cy - 1)[:, None, None]))
    add = numpy.where(valid & (photons > 0), photons * norm[:, None, None], 0.0)
    px_i = numpy.minimum(fx0[:, None] + kx[None, :], nw - 1)
    px_j = numpy.minimum(fy0[:, None] + ky[None, :], nh - 1)
    flat = px_i[:, :, None] * nh + px_j[:, None, :]
    image += numpy.bincount(flat.ravel(), weights=add.ravel(),
                            minlength=nw * nh).reshape(nw, nh)


def depth_keys(depth, cutoff_depth=1000.0e-9, res=PSF_RES):
    """``psf_depth_key`` (``_epifm.py:76-88``) for an array of depths."""
    d = numpy.abs(numpy.asarray(depth, dtype=float))
    inside = d < cutoff_depth + res
    keys = numpy.full(d.shape, -1, dtype=numpy.int64)
    keys[inside] = (d[inside] / res).astype(numpy.int64)
    return keys


def _radial_table(kind, depth_value, wavelength, sigma, na, r):
    if kind == "Gaussian":
        return gaussian_radial(r, sigma)
    return born_wolf_radial(r, depth_value, wavelength, na)


def _splat_keys(job):
    """Worker: footprints of every record of the given depth keys, one key at a time."""
    (nw, nh, px, kind, wavelength, sigma, na, radial_cutoff, depth_cutoff, res, groups) = job
    geom = QuadrantGeometry(radial_cutoff, res)
    image = numpy.zeros((nw, nh))
    for key, x, y, norm in groups:
        depth_value = depth_cutoff if key < 0 else key * res
        gq = quadrant_prefix(geom, _radial_table(kind, depth_value, wavelength, sigma, na, geom.r))
        splat_records(image, gq, geom.n, x, y, norm, px, res)
    return image


def frame_records(params, input_data, draws, frame_index=0, start_time=0.0, exposure_time=None,
                  states=None):
    """Physics of one frame, vectorised over particles (``_epifm.py:1121-1216``, ``:1267-1333``).

    Returns (records, optinfo, exposure_time): records are arrays (depth, x, y,
    norm) over every (sub-step, particle) with norm > 0, in the reference's
    order (sub-step, then particle); optinfo is the true_data dict.
    ``states`` is the bleaching budget dict (updated in place), as in
    ``epifm.output_frame``; ``draws.bleaching_time(m_id, beta)`` gives a new
    molecule's bleaching time.  Molecule ids must be unique within a sub-step
    (as ``sample_inputs`` makes them): a sub-step's budgets are updated
    together.
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

    p_0 = numpy.asarray(params.focal_point, dtype=float)
    nw, nh = params.image_size
    px = params.px
    amplitude0, penetration = snells_law(params.flux_density, params.source_wavelength,
                                         params.angle)
    n_emit0 = emit_photons(amplitude0, 1.0, params.abs_coeff, params.qy, params.radius)
    beta = params.half_life / numpy.log(2.0) if params.bleach_switch else None
    coeff = params.fluoem_norm_sum * params.psf_normalization
    recs = []
    acc = {}
    order = []
    for i, (i_time, particles) in enumerate(frame_data):
        current = i_time if i != 0 else t
        nxt = frame_data[i + 1][0] if i + 1 < len(frame_data) else t + exposure_time
        unit_time = nxt - current
        if unit_time < 1e-13:
            continue
        parts = numpy.asarray(particles, dtype=float)
        m_ids = parts[:, 3].astype(numpy.int64)
        p_state = parts[:, 4].copy()
        rel = parts[:, :3] - p_0[None, :]
        depth = rel[:, 0]
        amplitude = amplitude0 * numpy.exp(-numpy.abs(depth) / penetration)
        n_emit = emit_photons(amplitude, unit_time, params.abs_coeff, params.qy, params.radius)
        if states is not None and params.bleach_switch:
            budget = numpy.empty(len(m_ids))
            for k, m in enumerate(m_ids.tolist()):
                if m not in states:
                    states[m] = photon_budget(n_emit0, draws.bleaching_time(m, beta))
                budget[k] = states[m]
            budget = budget - n_emit
            gone = budget <= 0
            budget[gone] = 0
            p_state[gone] = 0.0
            for m, b in zip(m_ids.tolist(), budget.tolist()):
                states[m] = b
        norm = coeff * (p_state * n_emit / (4.0 * numpy.pi))
        live = norm > 0.0
        recs.append((depth[live], rel[live, 1], rel[live, 2], norm[live]))
        rows = numpy.stack([numpy.full(len(m_ids), unit_time), unit_time * p_state,
                            unit_time * parts[:, 1], unit_time * parts[:, 2],
                            unit_time * parts[:, 1], unit_time * parts[:, 2],
                            unit_time * depth, norm], axis=1)
        for m, row in zip(m_ids.tolist(), rows):
            if m not in acc:
                acc[m] = numpy.zeros(8)
                order.append(m)
            acc[m] += row
    optinfo = {}
    for m in order:
        v = acc[m]
        v[1] /= exposure_time
        v[2:6] /= v[0]
        v[2] = (v[2] - p_0[1]) / px + (nw - 1) * 0.5
        v[3] = (v[3] - p_0[2]) / px + (nh - 1) * 0.5
        optinfo[m] = v
    if recs:
        depth, x, y, norm = (numpy.concatenate(c) for c in zip(*recs))
    else:
        depth = x = y = norm = numpy.zeros(0)
    return (depth, x, y, norm), optinfo, exposure_time


def splat_frame(params, records, pool=None, workers=1):
    """FP64 expected photons (nw, nh) of a frame's records, grouped by depth key."""
    depth, x, y, norm = records
    nw, nh = params.image_size
    keys = depth_keys(depth, params.depth_cutoff)
    uniq = numpy.unique(keys)
    order = numpy.argsort(keys, kind="stable")
    bounds = numpy.searchsorted(keys[order], uniq, side="left").tolist() + [len(keys)]
    groups = [(int(k), x[order[a:b]], y[order[a:b]], norm[order[a:b]])
              for k, a, b in zip(uniq.tolist(), bounds[:-1], bounds[1:])]
    common = (nw, nh, params.px, params.fluorophore_type, params.psf_wavelength,
              params.radial_width, params.psf.na, params.radial_cutoff, params.depth_cutoff,
              PSF_RES)
    if pool is None or workers <= 1 or len(groups) < 2:
        return _splat_keys(common + (groups,))
    chunks = [groups[w::workers] for w in range(workers)]
    parts = pool.map(_splat_keys, [common + (c,) for c in chunks if c])
    return numpy.sum(parts, axis=0)


def output_frame_fast(params, input_data, draws, frame_index=0, start_time=0.0,
                      exposure_time=None, states=None, pool=None, workers=1, camera=True):
    """``epifm.output_frame`` for many emitters: the same camera array and infodict.

    With ``camera=False`` only the expectation channel is filled (no draws are
    taken for the detector).  ``pool`` (a spawned process pool of ``workers``
    processes) spreads the depth keys over processes.
    """
    records, optinfo, exposure_time = frame_records(params, input_data, draws, frame_index,
                                                    start_time, exposure_time, states)
    photons = splat_frame(params, records, pool, workers)
    nw, nh = params.image_size
    cam = numpy.zeros((nw, nh, 2))
    if params.background_switch:
        photons += params.background_mean
    expected = params.qe * photons
    cam[:, :, 0] = expected
    if camera:
        d = draws.camera(params, expected)
        cam[:, :, 1] = adc_counts(d["signal"] + d["noise"], params.fullwell, params.gain,
                                  params.offset, params.bit)
    info = dict(true_data=optinfo)
    if states is not None:
        info["fluorescence_states"] = dict(states)
    return cam, info
