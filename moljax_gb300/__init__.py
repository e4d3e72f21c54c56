"""moljax_gb300: GB300-native (sm_103a) method-of-lines step path with moljax's API.

The compute path is the native library ``_lib/libmoljax_gb300.so`` (CUDA C++,
C ABI in ``include/moljax_gb300.h``) called through ctypes with torch CUDA
tensors as the device buffers.  There is no CPU or library fallback.
"""

from moljax_gb300.core import *  # noqa: F401,F403
from moljax_gb300.core import autotune  # noqa: F401


__version__ = "0.1.0"
