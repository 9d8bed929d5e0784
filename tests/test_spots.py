"""Spot detection (the reference's analysis/spot_detection.py).

CPU: the oracle's fits against golden rows recorded from the reference
itself (tests/golden/make_spot_golden.py), and the Laplacian-of-Gaussian
filter against scipy.ndimage.gaussian_laplace.  GPU: every blob's fit from
``sc_spot_fit`` against the oracle's fits run to machine precision, and, for
the well-determined spots, against the reference's rows; blob detection and
fitting end to end on a synthetic image.
"""

import os

import numpy
import pytest

from oracle import spots as S

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def golden():
    return numpy.load(os.path.join(HERE, "golden", "spot_goldens.npz"))


@pytest.mark.parametrize("roi", [6, 4])
def test_oracle_matches_reference(golden, roi):
    import scipy
    if str(golden["versions"][1]) != scipy.__version__:
        pytest.skip("the goldens pin scipy %s's least_squares path" % golden["versions"][1])
    got = S.spot_detection(golden["image"], roi, golden["blobs"])
    numpy.testing.assert_array_equal(got, golden["roi%d_spots" % roi])


def test_log_kernels_match_scipy():
    """The Gaussian and second-derivative kernels the LoG kernel is given are
    scipy.ndimage's: separable 'reflect' correlations with them equal
    gaussian_laplace."""
    import scipy.ndimage as ndi
    from scopyon_gb300 import analysis as A
    img = numpy.random.RandomState(0).rand(37, 23)
    for s in (1.0, 2.5, 9.0, 30.0):
        phi, d2 = A._gauss_kernels(s)
        c = ndi.correlate1d
        lap = (c(c(img, d2, 0, mode="reflect"), phi, 1, mode="reflect") +
               c(c(img, phi, 0, mode="reflect"), d2, 1, mode="reflect"))
        ref = ndi.gaussian_laplace(img, s)
        assert numpy.abs(lap - ref).max() <= 1e-12 * numpy.abs(ref).max()


@pytest.mark.gpu
def test_gpu_log_cube_matches_scipy():
    """sc_log_cube against scipy.ndimage.gaussian_laplace (times -sigma^2),
    including kernels wider than the image (repeated reflection)."""
    import scipy.ndimage as ndi
    from scopyon_gb300 import _build
    _build.build()
    from scopyon_gb300 import analysis as A
    img = numpy.random.RandomState(0).rand(37, 23) * 100.0
    sigmas = numpy.array([1.0, 2.5, 9.0, 30.0])
    cube = A.log_cube(img, sigmas).cpu().numpy()
    for k, s in enumerate(sigmas):
        ref = -ndi.gaussian_laplace(img, s) * s * s
        assert numpy.abs(cube[:, :, k] - ref).max() <= 1e-12 * numpy.abs(ref).max()


@pytest.mark.gpu
def test_gpu_log_peaks_match_maximum_filter():
    """sc_log_peaks finds exactly the cells a 3 x 3 x 3 maximum filter (edges
    ignored) and the threshold select, on the GPU's own scale space."""
    import scipy.ndimage as ndi
    import torch
    from scopyon_gb300 import _build
    _build.build()
    from scopyon_gb300 import analysis as A
    from scopyon_gb300._lib import call, ptr, stream_ptr
    rng = numpy.random.RandomState(3)
    img = rng.poisson(5.0, (96, 80)).astype(float)
    X, Y = numpy.indices(img.shape)
    for cx, cy, a in ((20, 30, 200), (50, 61, 120), (80, 12, 90), (51, 63, 60)):
        img += a * numpy.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / 6.0)
    sigmas = numpy.linspace(1, 5, 6)
    cube = A.log_cube(img, sigmas)
    nw, nh, ns = cube.shape
    for threshold in (0.5, 5.0, 40.0):
        count = torch.zeros(1, dtype=torch.int32, device="cuda")
        found = torch.empty(3 * nw * nh * ns, dtype=torch.int32, device="cuda")
        call("sc_log_peaks", ptr(cube), nw, nh, ns, threshold, ptr(count), ptr(found),
             nw * nh * ns, stream_ptr())
        n = int(count.item())
        got = found[: 3 * n].view(n, 3).cpu().numpy()
        got = got[numpy.lexsort((got[:, 2], got[:, 1], got[:, 0]))]
        c = cube.cpu().numpy()
        mx = ndi.maximum_filter(c, size=3, mode="constant", cval=-numpy.inf)
        ref = numpy.argwhere((c == mx) & (c > threshold))
        numpy.testing.assert_array_equal(got, ref)
        assert n > 0


def test_prune_keeps_the_larger_of_overlapping_blobs():
    from scopyon_gb300 import analysis as A
    b = numpy.array([[10.0, 10.0, 3.0], [11.0, 10.0, 2.0], [40.0, 40.0, 2.0]])
    kept = A._prune(b, 0.5)
    numpy.testing.assert_array_equal(kept, b[[0, 2]])


def _well_determined(row, roi):
    return row[4] > 50 and 0.5 < row[5] < 3 * roi


@pytest.mark.gpu
@pytest.mark.parametrize("roi", [6, 4])
def test_gpu_fits_match_converged_oracle(golden, roi):
    from scopyon_gb300 import _build
    _build.build()
    from scopyon_gb300 import analysis
    img, blobs = golden["image"], golden["blobs"]
    fits = analysis.spot_fits(img, blobs, roi)
    checked = 0
    for b, f in zip(blobs, fits):
        ref = S.spot_fit(img, b, roi, tight=True)
        if ref is None or not _well_determined(ref, roi):
            continue
        assert f[6] == 0, (b, f)
        ref = numpy.array(ref)
        numpy.testing.assert_allclose(f[:2], ref[:2], rtol=0, atol=1e-6)
        numpy.testing.assert_allclose(f[2:6], ref[2:6], rtol=1e-6)
        checked += 1
    assert checked >= 10
    # regions that sum to <= 0 are skipped, as the reference skips them
    dark = analysis.spot_fits(numpy.zeros((20, 20)), [[10.0, 10.0, 2.0]], roi)
    assert dark[0, 6] == 1


@pytest.mark.gpu
@pytest.mark.parametrize("roi", [6, 4])
def test_gpu_spots_match_reference_where_well_determined(golden, roi):
    from scopyon_gb300 import _build
    _build.build()
    from scopyon_gb300 import analysis
    img, blobs = golden["image"], golden["blobs"]
    fits = analysis.spot_fits(img, blobs, roi)
    ref_rows = golden["roi%d_spots" % roi]
    # the reference's rows in blob order: match each to its blob's fit
    kept = fits[fits[:, 6] == 0]
    for row in ref_rows:
        if not _well_determined(row, roi):
            continue
        k = numpy.argmin(numpy.hypot(kept[:, 0] - row[0], kept[:, 1] - row[1]))
        got = kept[k]
        assert abs(got[0] - row[0]) < 2e-3 and abs(got[1] - row[1]) < 2e-3, (got, row)
        numpy.testing.assert_allclose(got[2:6], row[2:6], rtol=1e-3)
    got = analysis.spot_detection(img, roi_size=roi, blobs=blobs)
    assert got.shape[1] == 6 and len(got) == (fits[:, 6] == 0).sum()


@pytest.mark.gpu
def test_blob_detection_and_fits_end_to_end():
    from scopyon_gb300 import _build
    _build.build()
    from scopyon_gb300 import analysis
    rng = numpy.random.RandomState(4)
    X, Y = numpy.indices((128, 96)).astype(float)
    img = 20.0 + rng.normal(0.0, 1.0, X.shape)
    truth = []
    for cx in (20.3, 60.7, 101.2):
        for cy in (18.6, 49.1, 77.4):
            img += 300.0 * numpy.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / 4.5)
            truth.append((cx, cy))
    truth = numpy.array(truth)
    blobs = analysis.blob_detection(img, min_sigma=1, max_sigma=4, num_sigma=7, threshold=20)
    assert len(blobs) >= len(truth)
    for cx, cy in truth:
        assert numpy.hypot(blobs[:, 0] - cx, blobs[:, 1] - cy).min() < 1.0
    spots = analysis.spot_detection(img, roi_size=6, min_sigma=1, max_sigma=4, num_sigma=7,
                                    threshold=20)
    for cx, cy in truth:
        assert numpy.hypot(spots[:, 0] - cx, spots[:, 1] - cy).min() < 0.1
