"""pyranda_gb300: pyranda's compact-operator path on one NVIDIA GB300.

The package keeps pyranda's user API (``pyrandaSim`` with ``EOM``, ``setIC``,
``rk4``, ``ddx``/``ddy``/``ddz``, ``filter``/``gfilter``, ``ring``; the
``pyrandaTimestep`` and ``pyrandaBC`` packages) and runs it on the GPU through
the C ABI of ``libpyranda_gpu.so`` (include/pyranda_gpu.h).
"""
from .pyranda import pyrandaSim, pyrandaVar, pyrandaEq, pyrandaRestart, defaultMeshOptions  # noqa: F401
from .pyrandaTimestep import pyrandaTimestep  # noqa: F401
from .pyrandaBC import pyrandaBC  # noqa: F401
from .pyrandaPackage import pyrandaPackage  # noqa: F401

__version__ = "0.1.0"
