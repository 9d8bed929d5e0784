"""Spot detection on the GPU: ``scopyon.analysis.spot_detection``.

``spot_detection(data, roi_size, blobs)`` has the reference's signature and
return (src/scopyon/analysis/spot_detection.py:143-173): one row
(center_x, center_y, intensity, bg, height, sigma) per blob whose fit is
kept, in blob order.  Every blob's planar background and Gaussian fit run on
the GPU at once (``sc_spot_fit``, a warp per blob).  The reference fits with
scipy's trust-region least squares and stops at a relative cost change of
1e-8; the fits here run Levenberg-Marquardt to a stalled step, so where the
reference's fit is well determined the two agree to its own tolerance, and
where it is not (a region without a spot) they may stop in different places.

``blob_detection`` is the Laplacian-of-Gaussian scale-space search the
reference takes from scikit-image (``blob_log``, :14-46): the scale-normalised
LoG of the image at ``num_sigma`` scales (``sc_log_cube``, FP64 separable
passes with scipy.ndimage's kernels and edges), maxima over 3 x 3 x 3
neighbourhoods above ``threshold`` (``sc_log_peaks``), overlapping blobs
pruned on the host.  It is written from the published method, not from
scikit-image (absent here).
"""

import math

import numpy
import torch

from . import _lib
from ._lib import call, ptr, stream_ptr

__all__ = ["spot_detection", "blob_detection", "spot_fits", "log_cube"]


def _device():
    return torch.device("cuda")


def spot_fits(data, blobs, roi_size=6):
    """Every blob's fit: (n, 8) rows (center_x, center_y, intensity, bg,
    height, sigma, status, 0); status 0 is a kept spot, 1 a region summing to
    <= 0, 2 a failed fit, 3 a centre outside the region."""
    blobs = numpy.asarray(blobs, dtype=float).reshape(-1, 3)
    data = numpy.asarray(data, dtype=float)
    if data.ndim != 2:
        raise ValueError("data must be a 2-D image")
    if len(blobs) == 0:
        return numpy.zeros((0, 8))
    dev = _device()
    img = torch.from_numpy(numpy.ascontiguousarray(data)).to(dev)
    b = torch.from_numpy(numpy.ascontiguousarray(blobs)).to(dev)
    out = torch.empty(len(blobs), 8, dtype=torch.float64, device=dev)
    call("sc_spot_fit", ptr(img), data.shape[0], data.shape[1], ptr(b), len(blobs),
         float(roi_size), ptr(out), stream_ptr())
    return out.cpu().numpy()


def spot_detection(data, roi_size=6, blobs=None, processes=None, **kwargs):
    """Spots in ``data`` (W x H), one row (center_x, center_y, intensity, bg,
    height, sigma) per kept blob; ``blobs`` (n x 3: x, y, r) defaults to
    ``blob_detection(data, **kwargs)``.  ``processes`` is accepted for the
    reference's signature; the fits run on the GPU."""
    del processes
    if blobs is None:
        blobs = blob_detection(data, **kwargs)
    res = spot_fits(data, blobs, roi_size)
    return res[res[:, 6] == 0][:, :6].copy()


def _gauss_kernels(sigma, truncate=4.0):
    """1-D Gaussian and second-derivative kernels of radius int(truncate sigma
    + 0.5), the Gaussian normalised to sum 1 (as scipy.ndimage builds them)."""
    radius = int(truncate * float(sigma) + 0.5)
    x = numpy.arange(-radius, radius + 1, dtype=float)
    phi = numpy.exp(-0.5 * (x / sigma) ** 2)
    phi /= phi.sum()
    d2 = phi * (x * x - sigma * sigma) / sigma ** 4
    return phi, d2


def log_cube(data, sigmas):
    """Scale-normalised LoG of ``data`` (W x H) at each of ``sigmas``: a
    W x H x len(sigmas) FP64 tensor on the GPU (``sc_log_cube``)."""
    data = numpy.asarray(data, dtype=float)
    if data.ndim != 2:
        raise ValueError("data must be a 2-D image")
    dev = _device()
    nw, nh = data.shape
    phis, d2s, off, rad = [], [], [], []
    o = 0
    for s in sigmas:
        phi, d2 = _gauss_kernels(s)
        phis.append(phi)
        d2s.append(d2)
        off.append(o)
        rad.append((len(phi) - 1) // 2)
        o += len(phi)
    ns = len(sigmas)

    def dev_t(a, dtype):
        return torch.as_tensor(numpy.ascontiguousarray(a), dtype=dtype, device=dev)

    img = dev_t(data, torch.float64)
    phi_t = dev_t(numpy.concatenate(phis), torch.float64)
    d2_t = dev_t(numpy.concatenate(d2s), torch.float64)
    off_t = dev_t(numpy.array(off, dtype=numpy.int32), torch.int32)
    rad_t = dev_t(numpy.array(rad, dtype=numpy.int32), torch.int32)
    sig_t = dev_t(numpy.asarray(sigmas, dtype=float), torch.float64)
    work = torch.empty(2 * nw * nh * ns, dtype=torch.float64, device=dev)
    cube = torch.empty((nw, nh, ns), dtype=torch.float64, device=dev)
    call("sc_log_cube", ptr(img), nw, nh, ptr(phi_t), ptr(d2_t), ptr(off_t), ptr(rad_t),
         ptr(sig_t), ns, ptr(work), work.numel() * 8, ptr(cube), stream_ptr())
    return cube


def blob_detection(data, min_sigma=1, max_sigma=50, num_sigma=10, threshold=0.2, overlap=0.5):
    """Blobs (n x 3: x, y, r = sigma sqrt 2) in ``data`` by the scale-normalised
    Laplacian of Gaussian (the reference's defaults)."""
    data = numpy.asarray(data, dtype=float)
    sigmas = numpy.linspace(min_sigma, max_sigma, num_sigma)
    cube = log_cube(data, sigmas)
    nw, nh, ns = cube.shape
    cap = nw * nh * ns
    count = torch.zeros(1, dtype=torch.int32, device=cube.device)
    found = torch.empty(3 * cap, dtype=torch.int32, device=cube.device)
    call("sc_log_peaks", ptr(cube), nw, nh, ns, float(threshold), ptr(count), ptr(found), cap,
         stream_ptr())
    n = int(count.item())
    if n == 0:
        return numpy.zeros((0, 3))
    peaks = found[: 3 * n].view(n, 3).cpu().numpy()
    peaks = peaks[numpy.lexsort((peaks[:, 2], peaks[:, 1], peaks[:, 0]))]  # (i, j, s) order
    blobs = numpy.column_stack([peaks[:, 0].astype(float), peaks[:, 1].astype(float),
                                sigmas[peaks[:, 2]]])
    blobs = _prune(blobs, overlap)
    blobs[:, 2] = blobs[:, 2] * math.sqrt(2)
    return blobs


def _prune(blobs, overlap):
    """Of two blobs whose circles (radius sigma sqrt 2) overlap by more than
    ``overlap`` of the smaller circle's area, keep the larger."""
    keep = numpy.ones(len(blobs), dtype=bool)
    r = blobs[:, 2] * math.sqrt(2)
    for i in range(len(blobs)):
        for j in range(i + 1, len(blobs)):
            if not (keep[i] and keep[j]):
                continue
            d = math.hypot(blobs[i, 0] - blobs[j, 0], blobs[i, 1] - blobs[j, 1])
            r1, r2 = r[i], r[j]
            if d > r1 + r2:
                continue
            small = min(r1, r2)
            if d <= abs(r1 - r2):
                frac = 1.0
            else:
                a1 = r1 * r1 * math.acos((d * d + r1 * r1 - r2 * r2) / (2 * d * r1))
                a2 = r2 * r2 * math.acos((d * d + r2 * r2 - r1 * r1) / (2 * d * r2))
                a3 = 0.5 * math.sqrt(max((-d + r1 + r2) * (d + r1 - r2) * (d - r1 + r2) *
                                         (d + r1 + r2), 0.0))
                frac = (a1 + a2 - a3) / (math.pi * small * small)
            if frac > overlap:
                if r1 > r2:
                    keep[j] = False
                else:
                    keep[i] = False
    return blobs[keep]
