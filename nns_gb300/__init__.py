"""nns_gb300 -- GB300-native Barnes-Hut gravity pipeline (libnbx.so + host mirror).

``nns_gb300.ic`` (initial conditions) is pure numpy.  ``nns_gb300.barnes_hut``
holds the host classes; it needs torch and the built libnbx.so and raises
ImportError when the library is missing -- there is no CPU fallback.
"""
from . import ic  # noqa: F401

__all__ = ["ic", "barnes_hut"]


def __getattr__(name):
    if name == "barnes_hut":
        from . import barnes_hut as bh
        return bh
    raise AttributeError(name)
