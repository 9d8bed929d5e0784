"""FP64 restatement of scopyon's spot fits (test infrastructure).

Follows src/scopyon/analysis/spot_detection.py:49-173 with scipy's
least_squares, as the reference does; ``tight=True`` runs the same fits to
machine precision (ftol = xtol = gtol = 1e-15), the optimum a fully
converged fit should reach.
"""

import numpy
import scipy.optimize

__all__ = ["spot_fit", "spot_detection"]


def _planar_background(roi, tol):
    """Plane a5 i + a6 j + a7 through the region's four edges (:61-78)."""
    m, n = roi.shape
    edge = roi[0, :-1].sum() + roi[-1, :-1].sum() + roi[:-1, 0].sum() + roi[:-1, -1].sum()
    a7_init = (edge - (roi[0, 0] + roi[0, -1] + roi[-1, 0] + roi[-1, -1])) / (2 * (m + n - 2))

    def error_func(p):
        a5, a6, a7 = p
        left = roi[0, :] - (numpy.arange(n) * a6 + a7)
        right = roi[-1, :] - ((m - 1) * a5 + numpy.arange(n) * a6 + a7)
        bottom = roi[:, 0] - (numpy.arange(m) * a5 + a7)
        top = roi[:, -1] - (numpy.arange(m) * a5 + (n - 1) * a6 + a7)
        return numpy.concatenate([left, right, bottom, top])

    res = scipy.optimize.least_squares(error_func, (0.0, 0.0, a7_init), **tol)
    return None if res.success <= 0 else res.x


def _gaussian(a1, a2, a3, a4):
    return lambda x, y: a1 * numpy.exp(-((x - a2) ** 2 + (y - a3) ** 2) / a4)


def spot_fit(data, blob, roi_size, tight=False):
    """One blob's row (center_x, center_y, intensity, bg, height, sigma), or
    None where the reference skips it (:105-132)."""
    tol = dict(ftol=1e-15, xtol=1e-15, gtol=1e-15) if tight else {}
    x, y, _ = blob
    x0, x1 = int(x - roi_size), int(x + roi_size) + 1
    y0, y1 = int(y - roi_size), int(y + roi_size) + 1
    x0, x1 = max(0, x0), min(data.shape[0], x1)
    y0, y1 = max(0, y0), min(data.shape[1], y1)
    roi = data[x0:x1, y0:y1]
    if roi.sum() <= 0:
        return None
    m, n = roi.shape
    plane = _planar_background(roi, tol)
    if plane is None:
        return None
    a5, a6, a7 = plane
    bg = (numpy.tile(numpy.arange(m)[:, None], (1, n)) * a5 +
          numpy.tile(numpy.arange(n), (m, 1)) * a6 + a7)
    rest = roi.astype(numpy.float64) - bg
    total = rest.sum()
    X, Y = numpy.indices(rest.shape)
    start = (255, (X * rest).sum() / total, (Y * rest).sum() / total, roi_size / 2)
    res = scipy.optimize.least_squares(
        lambda p: numpy.ravel(_gaussian(*p)(*numpy.indices(rest.shape)) - rest), start, **tol)
    if res.success <= 0:
        return None
    h, cx, cy, s = res.x
    if not (0 <= cx < m and 0 <= cy < n):
        return None
    inten = _gaussian(*res.x)(*numpy.indices(roi.shape)).sum()
    return (cx + x0, cy + y0, inten, bg.sum(), h, s)


def spot_detection(data, roi_size, blobs, tight=False):
    rows = [spot_fit(data, b, roi_size, tight) for b in blobs]
    return numpy.array([r for r in rows if r is not None])
