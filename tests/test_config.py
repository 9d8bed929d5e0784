"""Configuration behaviour, mirroring the reference's test/test_config.py."""

import numpy
import pytest

from scopyon_gb300 import _yaml
from scopyon_gb300.config import (Configuration, DefaultConfiguration, DimensionalityError,
                                  Quantity)


def test_default_loads():
    config = DefaultConfiguration()
    assert config.default.type == "epifm"
    assert config.get("method") == "default"


def test_get_set():
    config = DefaultConfiguration()
    assert config.default.detector.exposure_time == pytest.approx(0.1)
    config.default.detector.exposure_time = 0.033
    assert config.default.detector.exposure_time == pytest.approx(0.033)


def test_update_plain_and_value_only():
    config = DefaultConfiguration()
    config.update("""
    default:
        detector:
            exposure_time: 0.033
    """)
    assert config.default.detector.exposure_time == pytest.approx(0.033)
    config.update("""
    default:
        detector:
            exposure_time:
                value: 0.1
    """)
    assert config.default.detector.exposure_time == pytest.approx(0.1)


def test_update_with_units():
    config = DefaultConfiguration()
    config.update("""
    default:
        detector:
            exposure_time:
                value: 0.033
                units: s
    """)
    assert config.default.detector.exposure_time == pytest.approx(0.033)
    config.update("""
    default:
        detector:
            exposure_time:
                value: 100
                units: ms
    """)
    with pytest.warns(UserWarning):
        assert config.default.detector.exposure_time == pytest.approx(0.1)
    config.default.detector.exposure_time = 0.033
    assert config.default.detector.exposure_time == pytest.approx(0.033)


def test_quantity_assignment_and_dimension_check():
    config = DefaultConfiguration()
    config.default.detector.exposure_time = Quantity(33, "ms")
    with pytest.warns(UserWarning):
        assert config.default.detector.exposure_time == pytest.approx(0.033)
    config = DefaultConfiguration()
    with pytest.raises(DimensionalityError):
        config.default.detector.exposure_time = Quantity(33, "m")


def test_refuses_dict_and_unknown_keys():
    config = DefaultConfiguration()
    with pytest.raises(TypeError):
        config.default.detector.exposure_time = {"value": 1}
    with pytest.raises(KeyError):
        config.default.detector.no_such_key = 1
    with pytest.raises(KeyError):
        config.default.no_such_tree


def test_units_to_si():
    cfg = Configuration(yaml={"a": {"value": 250, "units": "nm"}, "b": {"value": 72, "units": "degree"},
                              "c": {"value": 4e5, "units": "W / m ** 2"},
                              "d": {"value": [1.0, 2.0], "units": "um"}})
    with pytest.warns(UserWarning):
        assert cfg.a == pytest.approx(250e-9)
        assert cfg.b == pytest.approx(numpy.deg2rad(72))
        assert cfg.d == pytest.approx([1e-6, 2e-6])
    assert cfg.c == 4e5


def test_yaml_subset():
    doc = _yaml.load("""
    # comment
    a: !!int 3
    b: [!!int 512, !!int 512]   # flow list
    c:
        d: "none"
        e: null
        f: true
        g: 16.0e-6
        h: kg / s ** 3
    l:
        - 1
        - two
    """)
    assert doc == {"a": 3, "b": [512, 512], "c": {"d": "none", "e": None, "f": True, "g": 16.0e-6,
                                                   "h": "kg / s ** 3"}, "l": [1, "two"]}
    with pytest.raises(ValueError):
        _yaml.load("a: [1, 2")


def test_save_roundtrip(tmp_path):
    config = DefaultConfiguration()
    path = tmp_path / "c.yaml"
    config.save(path)
    again = Configuration(filename=str(path))
    assert again.yaml == config.yaml
