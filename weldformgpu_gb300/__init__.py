"""GB300-native explicit SPH solid-mechanics step (WeldFormGPU's hot path).

The compute path is libweldform_gb300.so (hand-written sm_103a CUDA kernels
behind the C ABI in include/weldform_gb300.h); this package is its host
binding.  `Domain_d` mirrors the reference's SPH::Domain_d.
"""
from . import _abi  # noqa: F401


def __getattr__(name):
    # lazy: importing the package must not require the CUDA library
    if name in ("Domain_d", "WeldformError", "lib", "version", "release_cache"):
        from . import domain
        return getattr(domain, name)
    raise AttributeError(name)
