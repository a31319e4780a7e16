"""The reference's base import path (pyhermes/base/__init__.py)."""
from ..projection import SFCProjection
from ..window import WindowFunc

__all__ = ["SFCProjection", "WindowFunc"]
