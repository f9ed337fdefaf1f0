"""Host-side binding of the GB300 FDTD engine (libfdtd_gb300.so)."""
from . import abi, spec, problems  # noqa: F401
