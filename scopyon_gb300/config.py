"""Configuration tree for the GB300 image-formation engine.

Mirrors ``scopyon.Configuration`` / ``scopyon.DefaultConfiguration``
(reference ``src/scopyon/config.py:26-165``): a nested mapping read from YAML,
attribute access into sub-trees, and ``{value, units}`` leaves returned as SI
magnitudes.  Assignments keep the reference's rules: plain values replace a
leaf (dropping its units), ``Quantity`` values are dimension-checked against
the leaf they replace, and dict values are refused.

Keys that only this engine reads live under ``<method>.gpu`` (see
``default.yaml``); the reference ignores unknown keys, so one file drives both.
"""

import collections.abc
import copy
import os
import pathlib
import warnings

from . import _yaml
from ._units import DimensionalityError, Quantity, parse_units, to_base_magnitude

__all__ = ["Configuration", "DefaultConfiguration", "Quantity", "DimensionalityError"]

_DEFAULT_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "default.yaml")


def dict_merge(dst, src):
    """Deep-merge ``src`` into ``dst`` in place (reference ``config.py:19-24``)."""
    for key, value in src.items():
        if isinstance(dst.get(key), dict) and isinstance(value, collections.abc.Mapping):
            dict_merge(dst[key], value)
        else:
            dst[key] = value


def _dump(tree, indent=0):
    lines = []
    pad = " " * indent
    for key, value in tree.items():
        if isinstance(value, dict):
            lines.append("%s%s:" % (pad, key))
            lines.extend(_dump(value, indent + 4))
        else:
            lines.append("%s%s: %s" % (pad, key, _dump_scalar(value)))
    return lines


def _dump_scalar(value):
    if value is None:
        return "null"
    if isinstance(value, bool):
        return "true" if value else "false"
    if isinstance(value, int):
        return "!!int %d" % value
    if isinstance(value, float):
        return repr(value)
    if isinstance(value, (list, tuple)):
        return "[" + ", ".join(_dump_scalar(v) for v in value) + "]"
    text = str(value)
    return '"%s"' % text.replace('"', '\\"')


class Configuration(collections.abc.Mapping):
    """Nested configuration with SI conversion of ``{value, units}`` leaves."""

    def __init__(self, filename=None, yaml=None):
        if filename is not None:
            if yaml is not None:
                raise ValueError("give either filename or yaml, not both")
            with open(str(filename)) as f:
                self.__yaml = _yaml.load(f.read())
        elif yaml is not None:
            if isinstance(yaml, str):
                yaml = _yaml.load(yaml)
            elif isinstance(yaml, Configuration):
                yaml = yaml.yaml
            self.__yaml = yaml
        else:
            self.__yaml = None

    @classmethod
    def from_reference(cls, config):
        """Wrap a ``scopyon.Configuration`` (anything with a ``.yaml`` tree)."""
        return cls(yaml=copy.deepcopy(config.yaml))

    def __repr__(self):
        return "\n".join(_dump(self.__yaml or {})) + "\n"

    def save(self, file):
        """Write the tree as YAML to ``file``."""
        if not isinstance(file, (str, pathlib.PurePath)):
            raise TypeError("a file name is required")
        with open(str(file), "w") as f:
            f.write(repr(self))

    def update(self, conf):
        """Deep-merge a Configuration, a dict or YAML text into this tree."""
        if isinstance(conf, Configuration):
            dict_merge(self.__yaml, conf.yaml)
        elif isinstance(conf, dict):
            dict_merge(self.__yaml, conf)
        elif hasattr(conf, "yaml") and isinstance(conf.yaml, dict):
            dict_merge(self.__yaml, conf.yaml)
        else:
            dict_merge(self.__yaml, _yaml.load(conf))

    @property
    def yaml(self):
        return self.__yaml

    def get(self, key, defaultobj=None):
        return self.__yaml.get(key, defaultobj)

    def __getitem__(self, key):
        return getattr(self, key)

    def __len__(self):
        return len(self.__yaml)

    def __iter__(self):
        return (key for key, value in self.__yaml.items()
                if not isinstance(value, dict) or "value" in value)

    def __contains__(self, key):
        return self.__yaml is not None and key in self.__yaml

    def __getattr__(self, key):
        if key.startswith("_"):
            raise AttributeError(key)
        tree = self.__yaml
        if tree is None or key not in tree:
            raise KeyError("'%s'" % key)
        value = tree[key]
        if isinstance(value, dict):
            if "value" not in value:
                return Configuration(yaml=value)
            if value["value"] is not None and "units" in value:
                factor, _ = parse_units(value["units"])
                if factor != 1.0:
                    warnings.warn("Unit conversion in '%s' from [%s] to SI base units"
                                  % (key, value["units"]))
                return to_base_magnitude(value["value"], value["units"])
            return value["value"]
        return value

    def __setattr__(self, key, value):
        if key.startswith("_"):
            object.__setattr__(self, key, value)
            return
        tree = self.__yaml
        if key not in tree:
            raise KeyError("'%s'" % key)
        if isinstance(value, dict):
            raise TypeError("The given value for '%s' has wrong type: %r" % (key, value))
        original = tree[key]
        if isinstance(original, dict) and "value" not in original:
            raise ValueError("Cannot update '%s'." % key)
        if isinstance(value, Quantity):
            if isinstance(original, dict) and "units" in original:
                if not value.check(original["units"]):
                    raise DimensionalityError(value.units, original["units"],
                                              value.dimensionality,
                                              parse_units(original["units"])[1])
            tree[key] = dict(value=value.magnitude, units=value.units)
        else:
            tree[key] = value


class DefaultConfiguration(Configuration):
    """The packaged default tree (same keys and values as scopyon's ``scopyon.yaml``)."""

    def __init__(self):
        with open(_DEFAULT_PATH) as f:
            Configuration.__init__(self, yaml=_yaml.load(f.read()))
