"""GB300-native volume renderer for Ascent's scene `volume` plot.

Layers:
  include/gvr.h, csrc/    C ABI + C++ host logic + sm_103a CUDA kernels (libgvr.so)
  _native, scene          ctypes binding and the device-resident Scene handle
  volume                  vtkh::VolumeRenderer host logic (samples, LUT, params)
  workloads               seeded synthetic inputs of the benchmark configurations
"""
from ._native import GvrError, Camera, RenderParams  # noqa: F401

__all__ = ["GvrError", "Camera", "RenderParams"]

from .ascent import Ascent, AscentError  # noqa: E402,F401

__all__ += ["Ascent", "AscentError"]
