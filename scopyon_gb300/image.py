"""Image wrapper returned by ``form_image`` / ``generate_images``.

Same core interface as ``scopyon.Image`` (reference src/scopyon/image.py:12-150):
``as_array``, ``as_8bit``, ``save`` (.npy / .csv).  Plotting and PNG/video
writing are outside this engine.
"""

import os

import numpy

__all__ = ["Image"]


class Image:

    def __init__(self, data):
        data = numpy.asarray(data)
        if not (data.ndim == 2 or (data.ndim == 3 and data.shape[2] == 3)):
            raise ValueError("an image is 2-D or RGB (H, W, 3)")
        self.__data = data

    @staticmethod
    def load(file):
        name = str(file)
        ext = os.path.splitext(name)[1].lower()
        if ext == ".npy":
            return Image(numpy.load(name))
        if ext == ".csv":
            return Image(numpy.loadtxt(name))
        raise ValueError("unsupported image file type %r" % ext)

    def as_array(self):
        return self.__data

    @property
    def shape(self):
        return self.__data.shape

    def as_8bit(self, cmin=None, cmax=None, low=None, high=None):
        """Linear rescale to uint8 (reference image.py:125-150)."""
        data = self.__data
        cmin = data.min() if cmin is None else cmin
        cmax = data.max() if cmax is None else cmax
        low = 0 if low is None else low
        high = 255 if high is None else high
        scale = (high - low) / (cmax - cmin) if cmax != cmin else 0.0
        out = (data - cmin) * scale + low
        return Image(numpy.clip(out, 0, 255).astype(numpy.uint8))

    def save(self, filename):
        name = str(filename)
        ext = os.path.splitext(name)[1].lower()
        if ext == ".npy":
            numpy.save(name, self.__data)
        elif ext == ".csv":
            numpy.savetxt(name, self.__data)
        else:
            raise ValueError("unsupported image file type %r (use .npy or .csv)" % ext)
