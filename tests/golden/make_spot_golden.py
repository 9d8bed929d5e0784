"""Golden spot fits from the reference's spot detection (given blobs).

Run here, where the reference source is mounted read-only:

    python tests/golden/make_spot_golden.py /root/reference/src

The reference's ``analysis/spot_detection.py`` needs only numpy and scipy when
the blobs are given (``blob_detection`` needs scikit-image, which is absent),
so the module is loaded from its file without the package's ``analysis``
import (whose HMM module needs hmmlearn).  A seeded synthetic image (planar
background, Gaussian spots, Gaussian noise, one dark patch) and its blobs go
in; the reference's ``spot_detection(data, roi_size, blobs)`` rows come out.
Writes ``spot_goldens.npz`` next to this file.
"""

import importlib.util
import os
import sys

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))


def synthetic_image(seed=17, nw=96, nh=80, n_spots=14):
    rng = numpy.random.RandomState(seed)
    X, Y = numpy.indices((nw, nh)).astype(float)
    img = 40.0 + 0.15 * X - 0.1 * Y
    truth = []
    for _ in range(n_spots):
        cx, cy = rng.uniform(8, nw - 8), rng.uniform(8, nh - 8)
        h, s2 = rng.uniform(80, 400), rng.uniform(2.0, 6.0)
        img += h * numpy.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / s2)
        truth.append((cx, cy, h, s2))
    img += rng.normal(0.0, 3.0, img.shape)
    img[70:86, 2:14] = 0.0  # a dark patch: its ROI sums to zero
    truth = numpy.array(truth)
    blobs = numpy.column_stack([numpy.rint(truth[:, 0] + rng.uniform(-1.5, 1.5, n_spots)),
                                numpy.rint(truth[:, 1] + rng.uniform(-1.5, 1.5, n_spots)),
                                numpy.full(n_spots, 2.0)])
    blobs = numpy.vstack([blobs, [[78.0, 7.0, 2.0],     # the dark patch
                                  [1.0, 40.0, 2.0],     # clipped by the image edge
                                  [94.0, 79.0, 2.0]]])  # a corner
    return img, truth, blobs


def main():
    src = sys.argv[1] if len(sys.argv) > 1 else "/root/reference/src"
    path = os.path.join(src, "scopyon", "analysis", "spot_detection.py")
    spec = importlib.util.spec_from_file_location("reference_spot_detection", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    out = {}
    img, truth, blobs = synthetic_image()
    for roi in (6, 4):
        spots = mod.spot_detection(img, roi_size=roi, blobs=blobs)
        out["roi%d_spots" % roi] = numpy.asarray(spots, dtype=float)
    import scipy
    out["versions"] = numpy.array([numpy.__version__, scipy.__version__])
    out["image"] = img
    out["truth"] = truth
    out["blobs"] = blobs
    numpy.savez_compressed(os.path.join(HERE, "spot_goldens.npz"), **out)
    print("wrote", os.path.join(HERE, "spot_goldens.npz"), {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
