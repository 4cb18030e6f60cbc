"""Host-side bindings of the GB300 FEST-3D explicit path (C ABI in
include/fest_gpu.h, CUDA sources in csrc/)."""
from . import abi  # noqa: F401
