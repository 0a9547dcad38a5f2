"""openpv_gb300 -- GB300-native (sm_103a) synaptic delivery and LCA update for OpenPV models.

The compute path is libpvgpu.so (openpv_gb300/csrc, C ABI in include/pvgpu.h).  This
package holds the build step and the ctypes binding used by the tests, bench and
drop-in harness.  There is no CPU fallback: without the built library, calls raise.
"""
from . import build  # noqa: F401

__all__ = ["build", "capi"]
