"""Ownership of C-ABI handles."""
from . import _lib


class Handle:
    """Owns one C-ABI object and destroys it when garbage collected."""

    __slots__ = ("ptr", "_destroy")

    def __init__(self, ptr, destroy_name):
        self.ptr = ptr
        self._destroy = getattr(_lib.lib(), destroy_name)

    def __del__(self):
        try:
            if self.ptr:
                self._destroy(self.ptr)
                self.ptr = None
        except Exception:
            pass
