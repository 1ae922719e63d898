"""`import gs` alias of msplat_gb300 (the module name the reference's README uses)."""
from msplat_gb300 import *  # noqa: F401,F403
from msplat_gb300 import __all__, __version__  # noqa: F401
