"""GB300-native extensive off-target search, a drop-in for BEguidedOFF's
``beguidedoff(mode="extensive")`` (beguidedoff/__init__.py:19-54).

Importing the package loads neither the native library nor any GPU state; the
finder loads ``_build/libbgo.so`` when it is constructed.
"""
from . import genome_converter
from .types import GuideInput

__all__ = ["beguidedoff", "beguidedofffast", "GuideInput", "genome_converter"]


def beguidedoff(*args, mode: str = "extensive", **kwargs):
    """Create an off-target finder; only ``mode="extensive"`` is provided."""
    mode = str(mode).lower()
    if mode == "extensive":
        from .finder import beguidedoff as _extensive

        return _extensive(*args, **kwargs)
    if mode == "fast":
        raise NotImplementedError(
            "mode='fast' (the CPU FM-index filter) is not part of this package; "
            "use the reference implementation for it.")
    raise ValueError(f"Unknown mode {mode!r}; expected 'extensive' or 'fast'.")


def beguidedofffast(*args, **kwargs):
    return beguidedoff(*args, mode="fast", **kwargs)
