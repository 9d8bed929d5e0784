"""Spectral catalog lookups needed by the image-formation path.

Only two catalog facts reach the per-frame path (reference
``src/scopyon/_epifm.py:822-869``): the PSF wavelength (the emission peak on
the 1-nm grid ``arange(min_wave_length, max_wave_length, 1 nm)``) and the sum
of the normalised emission spectrum (``fluoem_norm``), which scales every
emitter's photon count.  The CMOS camera model also needs the tabulated
readout-noise distribution ``catalog/detector/RNDist_F40.csv``
(``_epifm.py:332-345``).

Lookup order: a catalog directory given by the caller (``gpu.catalog_dir``),
then the catalog of an installed ``scopyon`` package, then, for fluorophore
peaks only, the table in ``_catalog_peaks.py`` (generated from the scopyon
catalog by ``_make_catalog_peaks.py``).
"""

import csv
import io
import os

import numpy

__all__ = ["find_catalog_dir", "read_catalog", "fluorophore_spectra", "psf_wavelength_and_norm",
           "cmos_noise_table"]


def find_catalog_dir(explicit=None):
    if explicit:
        return explicit
    try:
        import importlib.util
        spec = importlib.util.find_spec("scopyon")
        if spec and spec.submodule_search_locations:
            for loc in spec.submodule_search_locations:
                cand = os.path.join(loc, "catalog")
                if os.path.isdir(cand):
                    return cand
    except (ImportError, ValueError):
        pass
    return None


def _isfloat(text):
    try:
        float(text)
        return True
    except ValueError:
        return False


def read_catalog(path):
    """Sections of a catalog CSV: five header lines, then ``key`` rows and data rows
    (the format read by ``src/scopyon/io.py:29-52``)."""
    with open(path) as f:
        text = f.read()
    stream = io.StringIO(text)
    for _ in range(5):
        stream.readline()
    reader = csv.reader(stream)
    first = next(reader)
    if len(first) != 1 or _isfloat(first[0]):
        raise RuntimeError("A catalog in invalid format was given [%s]" % path)
    key, out = first[0], {}
    for row in reader:
        if len(row) == 1 and not _isfloat(row[0]):
            key = row[0]
        elif len(row) != 0:
            out.setdefault(key, []).append(row)
    return out


def _efficiency(rows, grid):
    """Spectrum on the 1-nm grid, integer-nm rows only (``_epifm.py:984-996``)."""
    data = numpy.array(rows, dtype=float)
    data = data[data[:, 0] % 1 == 0, :]
    eff = numpy.zeros(len(grid))
    nm = numpy.round(grid / 1e-9).astype(int)
    idx1 = numpy.isin(nm, data[:, 0])
    idx2 = numpy.isin(data[:, 0], nm)
    eff[idx1] = data[idx2, 1]
    return eff


def fluorophore_spectra(name, catalog_dir, min_wl=300e-9, max_wl=1000e-9):
    """(psf_wavelength, sum of normalised emission) from a fluorophore CSV."""
    grid = numpy.arange(min_wl, max_wl, 1e-9, dtype=float)
    sections = read_catalog(os.path.join(catalog_dir, "fluorophore", "%s.csv" % name))
    em = _efficiency(sections["Emission"], grid)
    index = int(em.argmax())
    em[index] = 100
    em /= sum(em)
    return grid[index], float(numpy.sum(em))


def psf_wavelength_and_norm(fluorophore, min_wl=300e-9, max_wl=1000e-9, wave_length=None,
                            catalog_dir=None, override=None):
    """PSF wavelength and emission-normalisation sum for a fluorophore config."""
    grid = numpy.arange(min_wl, max_wl, 1e-9, dtype=float)
    if fluorophore == "Gaussian":
        if wave_length is None:
            raise ValueError("fluorophore.wave_length must be given for a Gaussian fluorophore")
        return grid[int(numpy.abs(grid - wave_length).argmin())], 1.0
    if override is not None:
        return float(override), 1.0
    cdir = find_catalog_dir(catalog_dir)
    if cdir and os.path.exists(os.path.join(cdir, "fluorophore", "%s.csv" % fluorophore)):
        return fluorophore_spectra(fluorophore, cdir, min_wl, max_wl)
    from ._catalog_peaks import PEAKS
    if fluorophore not in PEAKS:
        raise ValueError("unknown fluorophore %r: give gpu.catalog_dir or gpu.psf_wavelength"
                         % fluorophore)
    peak_nm, norm_sum = PEAKS[fluorophore]
    index = peak_nm - int(round(min_wl / 1e-9))
    if not 0 <= index < len(grid):
        raise ValueError("emission peak %d nm outside the wavelength grid" % peak_nm)
    default_grid = abs(min_wl - 300e-9) < 1e-15 and abs(max_wl - 1000e-9) < 1e-15
    return grid[index], (norm_sum if default_grid else 1.0)


def cmos_noise_table(catalog_dir=None):
    """(values, probabilities) of the CMOS additive readout noise (RNDist_F40)."""
    cdir = find_catalog_dir(catalog_dir)
    path = os.path.join(cdir, "detector", "RNDist_F40.csv") if cdir else None
    if not path or not os.path.exists(path):
        raise FileNotFoundError(
            "the CMOS 'table' noise model needs scopyon's catalog/detector/RNDist_F40.csv: "
            "install scopyon, set gpu.catalog_dir, or use gpu.cmos_noise: scmos")
    return numpy.loadtxt(path, delimiter=",")
