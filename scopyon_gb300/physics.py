"""Host-side optics constants (FP64), evaluated once per configuration.

Same formulas and operation order as the reference so that every per-particle
quantity the kernels derive from them is the reference's to the last bit.
"""

import numpy

# CODATA 2018 exact values (the reference takes them from pint,
# src/scopyon/constants.py:12-17)
N_A = 6.02214076e23
HC = 6.62607015e-34 * 299792458

__all__ = ["N_A", "HC", "snells_law", "absorption_terms", "emit_photons"]


def snells_law(flux_density, source_wavelength, angle):
    """(amplitude, penetration depth) of the illumination (_epifm.py:1362-1428).

    EPI when sin^2(theta) / (n2/n1)^2 < 1: amplitude N_0 and infinite depth;
    TIRF otherwise: the evanescent s/p amplitudes of fused silica (n1 = 1.46)
    over a cell (n2 = 1.384) and depth lambda / (4 pi sqrt(n1^2 sin^2 - n2^2)).
    """
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
    return ((a2_x + a2_z) + a2_y) / 2, source_wavelength / (
        4.0 * numpy.pi * numpy.sqrt(n1 ** 2 * sin2 - n2 ** 2))


def absorption_terms(abs_coeff, radius):
    """(cross-section, absorbed fraction 1 - 10^-A) of get_emit_photons (_epifm.py:1344-1360)."""
    x_sec = numpy.log(10) * abs_coeff * 0.1 / N_A
    volume = (4.0 / 3.0) * numpy.pi * numpy.power(radius, 3)
    depth = 2.0 * radius
    a = (abs_coeff * 0.1 / N_A) * (1.0 / volume) * depth
    return x_sec, (1.0 - numpy.power(10.0, -a))


def emit_photons(amplitude, unit_time, x_sec, qy, beer):
    """Photons emitted in ``unit_time`` at the given excitation amplitude."""
    n_abs = amplitude * x_sec * unit_time
    return qy * n_abs * beer
