"""GB300-native DAWN frontier path: Python bindings over the C ABI.

The compute lives in ``lib/libdawn_gb300.so`` (hand-written sm_103a CUDA
behind the ``extern "C"`` entry points of ``include/dawn_gb300.h``).  This
package only loads that library with ctypes, converts numpy arrays to plain
pointers and turns status codes into exceptions.  It has no CPU fallback:
if the library is missing, importing :mod:`dawn_gb300.abi` raises.
"""

import os

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT_DIR = os.path.dirname(PKG_DIR)
LIB_DIR = os.path.join(ROOT_DIR, "lib")
BIN_DIR = os.path.join(ROOT_DIR, "bin")
CSRC_DIR = os.path.join(ROOT_DIR, "csrc")
HOST_DIR = os.path.join(ROOT_DIR, "host")
REPO_DIR = os.path.dirname(ROOT_DIR)
INCLUDE_DIR = os.path.join(REPO_DIR, "include")

__all__ = ["PKG_DIR", "ROOT_DIR", "LIB_DIR", "BIN_DIR", "CSRC_DIR", "HOST_DIR",
           "REPO_DIR", "INCLUDE_DIR"]
