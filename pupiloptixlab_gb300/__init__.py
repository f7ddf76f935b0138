"""GB300-native wavefront path tracer: a drop-in for PupilOptixLab's
"path tracing with MIS" pass.

Layers:
  include/pt_api.h         C-ABI (the drop-in boundary)
  csrc/                    CUDA kernels (sm_103a) and the host side of the ABI
  abi.py                   ctypes mirror of the ABI and the library loader
  scenes.py                scene builder, materials, procedural scenes
  api.py                   Python host wrapper (device buffers via torch)
  host_api.py              ctypes access to the C++ host layer (host/: mitsuba
                           XML/OBJ/HAIR loader, Pass / System / BufferManager
                           mirror of the reference's pass API, WavefrontPTPass)
  denoiser.py              learned U-Net denoiser (training and inference)
  denoise_data.py          training pairs rendered by the tracer
"""
from . import abi  # noqa: F401

__all__ = ["abi"]
