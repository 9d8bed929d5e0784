"""GB300-native image-formation engine with scopyon's API.

A drop-in for ``scopyon.form_image`` / ``scopyon.generate_images``: Brownian
emitters, photobleaching, PSF splatting and the EMCCD / CCD / CMOS camera
models run as CUDA kernels for sm_103a (``libscopyon_gb300.so``, C ABI in
``include/scopyon_gb300.h``); Python handles configuration and bookkeeping.
"""

from .config import Configuration, DefaultConfiguration, Quantity, DimensionalityError
from .image import Image
from .base import (EPIFMSimulator, EnvironSettings, InjectedDraws, create_simulator, form_image,
                   generate_images)
from .sampling import DeviceTrajectories, concatenate, sample_inputs, sample_points
from . import analysis, sampling2
from .sampling2 import StateTrajectories, sample

__all__ = ["Configuration", "DefaultConfiguration", "Quantity", "DimensionalityError", "Image",
           "EPIFMSimulator", "EnvironSettings", "InjectedDraws", "create_simulator", "form_image",
           "generate_images", "sample_inputs", "sample_points", "DeviceTrajectories",
           "concatenate", "sample", "sampling2", "StateTrajectories", "analysis"]

__version__ = "0.1.0"
