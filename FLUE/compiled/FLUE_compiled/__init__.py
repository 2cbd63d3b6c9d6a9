"""Stand-in for the f2py extension module ``FLUE_compiled``
(python/meson.build:55-67), whose Fortran module ``flue_c`` is exposed as
the submodule of the same name."""
from . import flue_c

__all__ = ["flue_c"]
