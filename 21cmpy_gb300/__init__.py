"""GB300-native excursion-set ionisation engine: a drop-in for 21cmpy's find_HII_bubbles and
delta_T programs, computed by hand-written sm_103a CUDA kernels behind a C ABI.

The package name starts with a digit, like the reference's own package; import it with
``importlib.import_module("21cmpy_gb300")``.
"""
from . import cosmology, grf, schedule  # noqa: F401

__all__ = ["cosmology", "grf", "schedule", "engine", "build_engine"]
__version__ = "0.1.0"


def build_engine(force: bool = False):
    """Compile the CUDA engine in-tree (nvcc, sm_103a) and return the library path."""
    from ._build import build
    return build(force=force)


def __getattr__(name):
    if name == "engine":
        import importlib
        return importlib.import_module(__name__ + ".engine")
    raise AttributeError(name)
