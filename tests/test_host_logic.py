"""Host-side bookkeeping of the engine against the oracle (CPU only)."""

import numpy
import pytest

import oracle as O
from scopyon_gb300 import _catalog, physics
from scopyon_gb300.base import EPIFMSimulator
from scopyon_gb300.config import DefaultConfiguration
from scopyon_gb300.epifm import EngineConfig, frame_windows


def test_physics_matches_goldens(golden):
    for angle, amp, pen, n1, n2 in golden["physics_rows"]:
        a, p = physics.snells_law(400000.0, 532e-9, angle)
        assert a == amp and p == pen
        x, b = physics.absorption_terms(83400, 20e-9)
        assert physics.emit_photons(a, 1.0, x, 0.61, b) == n1


def test_catalog_peaks(golden):
    for tag, name in (("tritc", "Tetramethylrhodamine(TRITC)"), ("egfp", "EGFP")):
        wl, norm = _catalog.psf_wavelength_and_norm(name)
        assert wl == golden["cat_%s_psf_wavelength" % tag]
        assert norm == golden["cat_%s_fluoem_norm_sum" % tag]


def test_gaussian_wavelength_grid():
    wl, norm = _catalog.psf_wavelength_and_norm("Gaussian", wave_length=6.0e-7)
    assert abs(wl - 6.0e-7) < 1e-15 and norm == 1.0


@pytest.mark.parametrize("fpn", ["none", "pixel", "column"])
def test_adc_maps_match_oracle(fpn):
    cfg = DefaultConfiguration()
    cfg.update({"default": {"detector": {"image_size": [6, 5]},
                            "analog_to_digital_converter": {"type": fpn, "count": 3.0,
                                                            "offset": 100, "bit": 12}}})
    eng = EngineConfig(cfg["default"], rng=numpy.random.RandomState(2))
    off, gain = O.adc_maps(6, 5, 12, 800000, 100, fpn, 3.0, numpy.random.RandomState(2))
    numpy.testing.assert_array_equal(eng.offset, off)
    numpy.testing.assert_array_equal(eng.gain, gain)


def test_depth_keys_match_oracle():
    cfg = DefaultConfiguration()
    eng = EngineConfig(cfg["default"])
    depths = numpy.array([0.0, 1e-9, 37e-9, -250.4e-9, 999e-9, 999.7e-9, 1000.5e-9, 1500e-9, -2e-6])
    keys = eng.depth_keys(depths)
    assert list(keys) == [O.psf_depth_key(d)[0] for d in depths]


def test_frame_windows_match_reference_semantics():
    times = numpy.arange(0, 21) * 0.5e-3
    w, exp = frame_windows(times, len(times), 0.0, 10e-3, 0)
    assert [i for i, _ in w] == list(range(20))
    assert all(abs(ut - 0.5e-3) < 1e-15 for _, ut in w)
    w, _ = frame_windows(times, len(times), 0.25e-3, 2e-3, 1)
    # t = 2.25 ms: starts inside the sample at 2.0 ms, first unit time is 0.25 ms
    assert w[0][0] == 4 and abs(w[0][1] - 0.25e-3) < 1e-15


@pytest.mark.parametrize("k", [2, 3, 4, 5])
def test_format_data_matches_oracle(k):
    rng = numpy.random.RandomState(k)
    inputs = rng.uniform(-1e-6, 1e-6, size=(7, k))
    if k >= 4:
        inputs[:, k - 2] = numpy.arange(7) + 3
        inputs[:, k - 1] = 1.0
    sim = EPIFMSimulator(DefaultConfiguration(), rng=numpy.random.RandomState(0))
    numpy.testing.assert_array_equal(sim._format_data(inputs), O.format_data(inputs))


def test_format_inputs_errors():
    sim = EPIFMSimulator(DefaultConfiguration(), rng=numpy.random.RandomState(0))
    with pytest.raises(ValueError):
        sim._format_data(numpy.zeros((3, 6)))
    with pytest.raises(ValueError):
        sim._format_inputs([(0.0, [1, 2])])
    with pytest.raises(TypeError):
        sim._format_inputs(3.0)


def test_unknown_detector_and_type():
    cfg = DefaultConfiguration()
    cfg.update({"default": {"detector": {"type": "PMT"}}})
    with pytest.raises(RuntimeError):
        EngineConfig(cfg["default"])
    cfg = DefaultConfiguration()
    cfg.update({"default": {"type": "lscm"}})
    with pytest.raises(ValueError):
        EngineConfig(cfg["default"])


@pytest.mark.parametrize("section,key,value", [
    ("detector", "image_size", [0, 64]), ("detector", "image_size", [64, 40000]),
    ("detector", "pixel_length", -16e-6), ("detector", "exposure_time", 0.0),
    ("detector", "QE", 1.5), ("analog_to_digital_converter", "bit", 0),
    ("analog_to_digital_converter", "bit", 40),
    ("analog_to_digital_converter", "fullwell", float("nan"))])
def test_corrupt_config_is_rejected_on_the_host(section, key, value):
    """A corrupt detector / ADC section raises ValueError before any launch."""
    cfg = DefaultConfiguration()
    cfg.update({"default": {section: {key: value}}})
    with pytest.raises(ValueError, match=key):
        EngineConfig(cfg["default"], rng=numpy.random.RandomState(0))


@pytest.mark.parametrize("value", [17, 256, -32])
def test_l2_fetch_hint_config_is_checked(value):
    """gpu.l2_fetch_bytes takes 0, 32, 64 or 128 (bytes); others raise ValueError."""
    cfg = DefaultConfiguration()
    assert EngineConfig(cfg["default"], rng=numpy.random.RandomState(0)).l2_fetch_bytes == 32
    cfg.update({"default": {"gpu": {"l2_fetch_bytes": value}}})
    with pytest.raises(ValueError, match="l2_fetch_bytes"):
        EngineConfig(cfg["default"], rng=numpy.random.RandomState(0))


def test_nvtx_ranges_config(monkeypatch):
    """NVTX ranges around the frame's launches are off by default and turned
    on by gpu.nvtx or by SCOPYON_GB300_NVTX=1."""
    monkeypatch.delenv("SCOPYON_GB300_NVTX", raising=False)
    cfg = DefaultConfiguration()
    assert EngineConfig(cfg["default"], rng=numpy.random.RandomState(0)).nvtx is False
    monkeypatch.setenv("SCOPYON_GB300_NVTX", "1")
    assert EngineConfig(cfg["default"], rng=numpy.random.RandomState(0)).nvtx is True
    monkeypatch.setenv("SCOPYON_GB300_NVTX", "0")
    cfg.update({"default": {"gpu": {"nvtx": True}}})
    assert EngineConfig(cfg["default"], rng=numpy.random.RandomState(0)).nvtx is True
