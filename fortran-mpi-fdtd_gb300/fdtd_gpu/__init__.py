"""Host-side binding of the GB300 FDTD engine (libfdtd_gb300.so)."""
from . import abi, spec, problems  # noqa: F401
from .job import Job, FdtdError, device_count, lib  # noqa: F401
from .serve import Server  # noqa: F401
