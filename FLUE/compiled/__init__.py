"""The compiled layer (python/FLUE/compiled/__init__.py:1-4): ``flue_c``."""
from .FLUE_compiled import flue_c

__all__ = ["flue_c"]
