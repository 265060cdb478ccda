"""Frame serializer, format-compatible with the reference's common/serializer."""
from .loader import Loader
from .saver import AsyncFrameSaver, Saver

__all__ = ["Saver", "Loader", "AsyncFrameSaver"]
